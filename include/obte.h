/*
 * obte.h — C ABI of the GB300 (sm_103a) phonon-BTE transport library.
 *
 * The reference (romanodev/OpenBTE) is pure Python; its transport path is the
 * pair of functions
 *     BTE_RTA(geo, mat, bcs, fourier, effective_thermal_conductivity, ...)   openbte/bte.py:19-271
 *     Fourier(geometry, thermal_conductivity, boundary_conditions, ...)      openbte/fourier.py:15-185
 * A Python FFI for that path (ctypes / cffi) binds the functions below; the
 * package's ``openbte_gb300.BTE_RTA`` / ``Fourier`` wrappers are exactly that
 * binding (openbte_gb300/_lib.py declares the prototypes).
 *
 * Conventions
 *   - every call returns an obte_status; obte_status_string() names it;
 *   - "host" arrays are read during the call only; "device" arrays are
 *     caller-owned CUDA device pointers (e.g. torch tensors) on the
 *     context's device; the library owns only its plans and scratch;
 *   - all work is issued on the stream given to obte_context_create and the
 *     call returns after that stream has finished the work it issued;
 *   - indices are 0-based int64, floating point is IEEE binary64 at the boundary.
 */
#ifndef OBTE_H
#define OBTE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  OBTE_OK = 0,
  OBTE_ERR_BAD_ARG = 1,           /* invalid size, index or pointer            */
  OBTE_ERR_OOM = 2,               /* device allocation failed                  */
  OBTE_ERR_ADMISSION = 3,         /* request exceeds the admitted HBM budget   */
  OBTE_ERR_NOT_CONVERGED = 4,     /* iteration cap reached before tolerance    */
  OBTE_ERR_CUDA = 5,              /* a CUDA runtime call failed                */
  OBTE_ERR_CYCLE = 6,             /* upwind graph has a cycle besides periodic */
  OBTE_ERR_UNSUPPORTED = 7,       /* input outside what the kernels implement  */
  OBTE_ERR_DEVICE_TIMEOUT = 8     /* a bounded device-side wait gave up        */
} obte_status;

typedef struct obte_context_s* obte_context;
typedef struct obte_plan_s* obte_plan;
typedef struct obte_fourier_plan_s* obte_fourier_plan;

/* Sweep precision.  OBTE_DOUBLE_FLOAT (sweeps only: obte_bte_sweep, obte_bte_sweep_fields) sweeps the FP64
 * tables in double-float arithmetic, pairs of FP32 numbers with ~44 significant bits computed on the FP32
 * pipe; it is the output pass of OBTE_FP32_REFINE solves. */
enum { OBTE_FP64 = 0, OBTE_FP32_REFINE = 1, OBTE_FP32 = 2, OBTE_DOUBLE_FLOAT = 3 };

/* Contact kinds for kappa_eff (openbte/bte.py:132-158). */
enum { OBTE_CONTACT_NONE = 0, OBTE_CONTACT_PERIODIC = 1, OBTE_CONTACT_MIXED = 2, OBTE_CONTACT_NANOWIRE = 3 };

/*
 * Problem description: the Mesh fields the transport path reads
 * (openbte/objects.py:244-268), with boundary-condition names already
 * resolved to side lists (openbte/objects.py:220-241).  All host arrays.
 */
typedef struct {
  int32_t dim;                    /* 2 or 3                                       */
  int64_t n_elems;
  int64_t n_sides;
  int32_t elem_nv;                /* sides per element (3 triangle, 4 tetrahedron) */
  const int64_t* side_elem_map;   /* [n_sides, 2]                                 */
  const double* normal_areas;     /* [n_sides, dim], outward from side_elem_map[:,0] */
  const double* elem_volumes;     /* [n_elems]                                    */
  const double* side_areas;       /* [n_sides]                                    */
  int64_t n_internal;
  const int64_t* internal;        /* [n_internal] sides coupling two elements (incl. kept periodic) */
  int64_t n_periodic;
  const int64_t* periodic_sides;  /* [n_periodic] kept periodic sides            */
  const double* periodic_jump;    /* [n_periodic] jump of their region           */
  int64_t n_diffuse;
  const int64_t* diffuse_sides;   /* [n_diffuse] diffuse (thermalising) walls     */
  int64_t n_mixed;
  const int64_t* mixed_sides;     /* [n_mixed] isothermal walls                   */
  const double* mixed_value;      /* [n_mixed] their temperature                  */
  int32_t contact_kind;           /* OBTE_CONTACT_*                               */
  int64_t n_contact;
  const int64_t* contact_sides;   /* [n_contact] (ignored for NANOWIRE)           */
  double contact_alpha;           /* jump (periodic) or value (mixed)             */
  double normalization;           /* EffectiveThermalConductivity.normalization   */
  int32_t is_nanowire;            /* BoundaryConditions.is_nanowire               */
  const double* heat_source;      /* [n_elems] or NULL (HeatSource data)          */
  /* Transmission-interface model (openbte/inverse/bte.py:145-163): fraction t in (0, 1] of the
   * inflow across each internal side that comes from the neighbour; NULL = 1 everywhere.  With
   * reflect_internal = 1 the rest, 1 - t, is the element's own outgoing flux at that side,
   * diffusely re-emitted (one reflected-temperature unknown per directed internal side, placed
   * after the diffuse walls in the T_B part of the state).                                     */
  const double* side_transmission;
  int32_t reflect_internal;
} obte_problem;

/* Ordinate data (openbte/objects.py:500-509). All host arrays. */
typedef struct {
  int32_t n_mfp;
  int32_t n_dir;
  int32_t dim_dir;                /* columns of vmfp                              */
  int32_t dim_sigma;              /* columns of sigma                             */
  const double* mfps;             /* [n_mfp] nm                                   */
  const double* vmfp;             /* [n_dir, dim_dir] unit directions             */
  const double* sigma;            /* [n_mfp, n_dir, dim_sigma]                    */
  const double* t_coeff;          /* [n_mfp, n_dir]                               */
  double heat_source_coeff;
} obte_material;

typedef struct {
  int32_t precision;              /* OBTE_FP64 | OBTE_FP32_REFINE | OBTE_FP32     */
  double rtol;                    /* residual tolerance ‖F(u)-u‖/‖u‖             */
  int32_t max_sweeps;             /* cap on transport sweeps                      */
  int32_t restart;                /* GMRES restart length                         */
  int32_t refine_steps;           /* FP64 residual corrections (FP32_REFINE)      */
  double inner_rtol;              /* inner FP32 tolerance (FP32_REFINE)           */
  int32_t warm_start;             /* 1: start from this plan's previous converged state (dT0 still
                                     fixes the conserved temperature level); 0: start from dT0 */
  int32_t precond;                /* periodic-inflow preconditioner (see obte_bte_precond_info):
                                     0 built on the plan's second solve (plans solved once do not pay
                                     its setup), 1 built on the first solve, -1 off; other values: 0.
                                     The environment variable OBTE_XPREC=0 / 1 overrides it. */
  int32_t dsa;                    /* diffusion-synthetic acceleration (no counterpart in the reference):
                                     1 on, -1 off, 0 (other values) on for problems with partially
                                     transmitting sides (side_transmission < 1), else off.
                                     OBTE_DSA=0 / 1 overrides it. */
} obte_solve_opts;

typedef struct {
  double kappa_eff;               /* sum of K                                    */
  int32_t n_sweeps;               /* transport sweeps issued                      */
  int32_t n_sweeps_fp64;          /* of which in FP64                             */
  double residual;                /* final ‖F(u)-u‖/‖u‖ (FP64)                   */
  double offset;                  /* constant shift applied to match the reference's conserved offset */
  int32_t converged;
  int32_t n_sweeps_df;            /* of which double-float output passes (FP32_REFINE, OBTE_REFINE_DF=1) */
} obte_solve_info;

/* ---- context ------------------------------------------------------------ */
/* stream: a cudaStream_t (NULL = legacy default stream). */
obte_status obte_context_create(int device, void* stream, obte_context* out);
obte_status obte_context_destroy(obte_context ctx);
obte_status obte_context_set_stream(obte_context ctx, void* stream);
const char* obte_status_string(int status);
/*
 * Device memory of destroyed plans is kept in a library-wide cache and reused by later plans instead of
 * being returned with cudaFree, which synchronises the whole device and stalls every solve running
 * on other streams (a serving loop drops a plan after every request).  The cache keeps at most
 * OBTE_DEVICE_CACHE_MB megabytes (default 16 GiB; older blocks beyond it are freed) and is trimmed by
 * itself when an allocation fails.  obte_device_cache_trim frees all of it (freed_bytes may be NULL);
 * obte_device_cache_bytes reports its size.  No counterpart in the reference (it has no device code).
 */
obte_status obte_device_cache_trim(int64_t* freed_bytes);
obte_status obte_device_cache_bytes(int64_t* cached_bytes);
/* Last error text recorded on this thread (CUDA error names, argument checks). */
const char* obte_last_error(void);
/* Number of kernel launches this library issued in the calling process (instrumentation). */
int64_t obte_launch_count(void);
/* Bytes this library copied host -> device for plan tables in the calling process (instrumentation). */
int64_t obte_h2d_bytes(void);

/* ---- BTE_RTA (openbte/bte.py:19-271) ------------------------------------ */
/*
 * Build the sweep plan: per-direction upwind level order with periodic faces
 * cut, shared-memory slot assignment for the live front, and the operator
 * tables of openbte/bte.py:47-158, uploaded to the device.  With ctx == NULL
 * the plan is host-only: its schedule can be queried but not solved.  Fails with
 * OBTE_ERR_CYCLE when a direction's upwind graph (periodic faces removed)
 * is not acyclic.
 */
obte_status obte_bte_plan_create(obte_context ctx, const obte_problem* prob,
                                 const obte_material* mat, obte_plan* out);
obte_status obte_bte_plan_destroy(obte_plan plan);
/*
 * New side transmissions [n_sides], each in (0, 1], for a plan created with side transmissions
 * (the transmission-interface model of inverse design).  Replaces openbte/inverse/bte.py:147-173
 * (get_rho_dependent: the transmission-dependent operator terms, recomputed per density field over
 * the density-independent geometry of bte.py:116-140).  The sweep order, slots and table layout do not
 * depend on t, so only the coefficients are recomputed and re-uploaded; the periodic-inflow
 * preconditioner is dropped, and the previous solution stays as the start of a warm-started solve (the
 * reference's design loop reuses it the same way, bte.py:234-236).  upload_bytes (may be NULL) receives
 * the bytes copied to the device.  OBTE_ERR_UNSUPPORTED for problems with isothermal walls or nanowire
 * terms (create a new plan), OBTE_ERR_BAD_ARG for a plan without side transmissions or a t outside (0, 1].
 */
obte_status obte_bte_plan_set_transmission(obte_plan plan, const double* side_transmission,
                                           int64_t* upload_bytes);
/*
 * Issue this plan's later work on `stream` (a cudaStream_t; work already issued is finished
 * first).  No counterpart in the reference: it lets a serving loop run plans concurrently on
 * separate streams.  One plan must not be used by two threads at the same time.
 */
obte_status obte_bte_plan_set_stream(obte_plan plan, void* stream);
/*
 * Do a solve's set-up ahead of it: pack and upload the device tables of the sweep precisions that
 * `precision` uses (OBTE_FP32_REFINE: FP32 and FP64) and allocate the solve scratch for GMRES
 * restart length `restart` (<= 0: 30).  obte_bte_solve does the same on first use; a serving loop
 * calls this on its host builder threads so that the GPU slot that later runs the solve only solves.
 * No counterpart in the reference, which builds its operators inside BTE_RTA (openbte/bte.py:47-185).
 */
obte_status obte_bte_plan_prepare(obte_plan plan, int32_t precision, int32_t restart);
/* Device bytes held by the plan (tables: their actual size once uploaded, an upper estimate before) and by
 * one solve's scratch (an upper estimate). */
obte_status obte_bte_plan_footprint(obte_plan plan, int32_t precision, int32_t restart,
                                    int64_t* plan_bytes, int64_t* solve_bytes);

/*
 * Source iteration to the fixed point (openbte/bte.py:193-256).
 *   dT0    device [n_elems]  initial lattice temperature (Fourier guess or zeros)
 *   dT     device [n_elems]  Temperature_BTE
 *   J      device [n_elems, dim_sigma]  Flux_BTE / 1e9 (W/m/nm), as accumulated by the reference
 *   K, S   device [n_mfp, n_dir]  per-ordinate kappa and suppression (aux)
 * OBTE_FP32_REFINE: GMRES with FP32 sweeps to inner_rtol, then an output pass that measures the true
 * residual and gives J, K, S, with FP32-swept corrections until the residual meets rtol.  The output pass
 * is FP64 below rtol = 5e-6; from 5e-6 up it is FP32 (its rounding, a few 1e-7 of the state, is under a
 * tenth of the tolerance), so a loose solve runs no FP64 sweep (OBTE_REFINE_FP64_PASS=1: FP64 always).
 */
obte_status obte_bte_solve(obte_plan plan, const obte_solve_opts* opts, const double* dT0,
                           double* dT, double* J, double* K, double* S, obte_solve_info* info);

/*
 * One transport sweep of every ordinate (precision: OBTE_FP64, OBTE_FP32 / OBTE_FP32_REFINE or
 * OBTE_DOUBLE_FLOAT) — the per-ordinate solves
 * A_mq T = B of openbte/bte.py:208-243 followed by the reduction of
 * openbte/objects.py:86-101 — at a given state.
 *   u_in   device [n_elems + n_diffuse + n_x]  (DeltaT, T_B, periodic inflow)
 *   u_out  device, same layout: (DeltaT', T_B', periodic outflow)
 *   with_source 0/1: include the perturbation (periodic jump, isothermal, nanowire, heat source)
 */
obte_status obte_bte_sweep(obte_plan plan, int32_t precision, const double* u_in, double* u_out,
                           int32_t with_source);
/*
 * The same sweep as obte_bte_sweep, with the same arguments and result, for
 * callers that cannot allocate device memory when they sweep: a host
 * framework that has reserved nearly all of the GPU's memory for its own pool
 * (where cudaMalloc fails or forces that pool to give memory back), or a
 * latency-bound loop where cudaMalloc / cudaFree would synchronise the device.
 * This call allocates nothing: its scratch (the per-sweep values, n_dir x
 * n_elems x 8 bytes in FP32 modes or x 16 in FP64, plus 288 bytes) lives in an
 * 8 MiB array inside the library, which every GPU that loads the library holds
 * until the process exits.  A larger problem is rejected with
 * OBTE_ERR_UNSUPPORTED (use obte_bte_sweep).  The plan's device tables for the
 * precision must already exist: building them allocates, so run obte_bte_sweep
 * or obte_bte_solve once in that precision at set-up, or this returns
 * OBTE_ERR_BAD_ARG.  The first call on a device looks up the array's device
 * address (once per device); make that first call before any stream capture.
 * All calls share the one array: calls whose GPU work overlaps (other threads,
 * other streams, other plans) race on it and must be serialised by the caller.
 * Each call synchronises the plan's stream before it returns.  The device address
 * looked up on the first call is kept for the life of the process: resetting
 * the device (cudaDeviceReset) after that first call is not supported.
 * No counterpart in the reference (it has no device code).
 */
obte_status obte_bte_sweep_static(obte_plan plan, int32_t precision, const double* u_in, double* u_out,
                                  int32_t with_source);
/*
 * One sweep like obte_bte_sweep that also stores every per-ordinate temperature: the solutions
 * T_mq = A_mq^-1 B_mq of openbte/bte.py:217-218, which the reference keeps inside its worker processes
 * and returns only reduced (ΔT, J, K, S).  For checks of single ordinates against exact solves, or for
 * callers that want the phonon temperatures themselves.
 *   T  device [n_dir, n_elems, n_mfp]: float for OBTE_FP32 / OBTE_FP32_REFINE, double for OBTE_FP64 and
 *      OBTE_DOUBLE_FLOAT
 * u_in, u_out and with_source as for obte_bte_sweep.
 */
obte_status obte_bte_sweep_fields(obte_plan plan, int32_t precision, const double* u_in, double* u_out,
                                  int32_t with_source, void* T);
/*
 * Test hook of the bounded device waits (no counterpart in the reference, whose Barrier.wait has no
 * timeout, openbte/objects.py:88-101): the plan's later sweeps do not issue the bulk copy of level
 * unit skip_unit of any direction (-1: none) and stop waiting for a unit's copy after wait_limit polls
 * (0: the default cap).  A sweep that reaches the skipped unit gives up, lets the copies it has in
 * flight land and returns OBTE_ERR_DEVICE_TIMEOUT; nothing faults or hangs, and the plan sweeps
 * normally again after (-1, 0).
 */
obte_status obte_bte_plan_test_wait_timeout(obte_plan plan, int32_t skip_unit, int32_t wait_limit);

/*
 * Inverse design: dkappa_eff/dt_s for every side of a plan created with side_transmission
 * (replaces compute_kappa_and_gradient, openbte/inverse/bte.py:27-95, for MFP-resolved
 * materials).  Solves like obte_bte_solve (same opts and dT0), keeps the per-ordinate
 * temperatures of the final sweep and evaluates the adjoint from them: the adjoint of
 * direction q is the forward solution of its reverse, so no second solve runs.
 *   grad_t  device [n_sides]; 0 on sides that are not internal.
 * Needs a direction set closed under reversal (else obte_bte_kappa_gradient_adjoint below),
 * sigma = a t_coeff mfp s (isotropic), the periodic jump only on the contact sides, and no
 * isothermal, heat-source or nanowire terms (else OBTE_ERR_UNSUPPORTED).  info->kappa_eff is
 * kappa_eff.
 */
obte_status obte_bte_kappa_gradient(obte_plan plan, const obte_solve_opts* opts, const double* dT0,
                                    double* grad_t, obte_solve_info* info);
/*
 * The same gradient for a direction set that is not closed under reversal: adjoint_plan is the plan's
 * problem (mesh, sides, transmissions, contact) with every direction reversed (ordinate q: -s_q, the same
 * t_coeff and MFP, sigma negated).  Its forward solve is the transposed transport of every ordinate, swept
 * in reverse order; its per-ordinate temperatures give the adjoint (lam_mq(c) = k V_c t_mq X'_mq(c)), so
 * the gradient costs two solves.  With sides that re-emit, sum_mq sigma_mq must be zero (else
 * OBTE_ERR_UNSUPPORTED); an adjoint plan that does not match returns OBTE_ERR_BAD_ARG.  After new
 * transmissions, update both plans.  adjoint_info (may be NULL) receives the adjoint solve's info.
 */
obte_status obte_bte_kappa_gradient_adjoint(obte_plan plan, obte_plan adjoint_plan, const obte_solve_opts* opts,
                                            const double* dT0, double* grad_t, obte_solve_info* info,
                                            obte_solve_info* adjoint_info);
/* Sizes of the state vector pieces: n_elems, n_diffuse, n_x. */
obte_status obte_bte_state_layout(obte_plan plan, int64_t* n_elems, int64_t* n_diffuse, int64_t* n_x);
/*
 * The cell diffusion operator of the plan's diffusion-synthetic acceleration (obte_solve_opts.dsa), as
 * built on the host (for inspection and tests; works on host-only plans): CSR over the elements, columns
 * sorted, volume-weighted and symmetric.  Call with row_ptr = col = val = NULL to get *nnz; then with
 * arrays of n_elems + 1 / *nnz / *nnz entries (*nnz = their capacity).  *project = 1 when the operator
 * has the constant null vector (no isothermal walls) and a solve projects its source to zero sum.
 */
obte_status obte_bte_dsa_operator(obte_plan plan, int64_t* nnz, int32_t* row_ptr, int32_t* col, double* val,
                                  int32_t* project);
/*
 * Periodic-inflow preconditioner of the plan (no counterpart in the reference, whose per-ordinate
 * sparse LU solves the periodic coupling directly): built when obte_solve_opts.precond asks for it (by
 * default on the plan's second solve).  n_blocks: ordinates it covers (0: none, or not built yet);
 * setup_sweeps: FP32 sweeps its setup ran (detection and probing); setup_ms: host wall time of the
 * setup.  Any pointer may be null.
 */
obte_status obte_bte_precond_info(obte_plan plan, int32_t* n_blocks, int32_t* setup_sweeps, double* setup_ms);
/*
 * Device memory of the plan's periodic-inflow preconditioner, for admission control: resident = bytes
 * the built preconditioner holds (0 when none was built; obte_bte_plan_footprint's plan_bytes include
 * them); build_bound = upper bound of the device bytes building it would allocate, resident blocks and
 * transient probe vectors together (0 once a build was tried, when the plan has no periodic inflow a
 * block could cover, or for a host-only plan).  Any pointer may be null.
 */
obte_status obte_bte_precond_bytes(obte_plan plan, int64_t* resident, int64_t* build_bound);
/*
 * Sweep schedule of direction q, as built on the host (for bit-exact checks):
 *   order  host [n_elems]      element processed at each position
 *   level_ptr host [n_levels+1] (pass NULL to query n_levels via *n_levels)
 */
obte_status obte_bte_schedule(obte_plan plan, int32_t q, int64_t* order, int64_t* level_ptr,
                              int64_t* n_levels, int64_t* n_slots);
/*
 * Operator coefficients of direction q in the sweep order of obte_bte_schedule, as built on the host
 * (openbte/bte.py:47-110 per ordinate direction; for bit-exact checks).  Any pointer may be NULL:
 *   in_coef host [n_elems * elem_nv]  inflow coefficients of each position (upwind faces, then walls;
 *                                     zero past the last inflow entry)
 *   D       host [n_elems]            outflow diagonal
 *   P       host [n_elems]            periodic jump source (and isothermal-wall / nanowire terms)
 */
obte_status obte_bte_schedule_coefficients(obte_plan plan, int32_t q, double* in_coef, double* D, double* P);
/*
 * 64-bit FNV-1a digest of the packed sweep tables (level units, per-item records, special entries, periodic
 * prefetch lists, output entries, contact coefficients and K shifts, wall outputs, periodic sources, wall
 * offset weights) that a plan uploads for `precision` (OBTE_FP64: FP64 tables, else FP32),
 * built on the host; works on host-only plans.  Two hosts or builds that pack the same plan identically
 * give the same digest.
 */
obte_status obte_bte_tables_digest(obte_plan plan, int32_t precision, uint64_t* digest);

/* ---- Fourier (openbte/fourier.py:15-185) -------------------------------- */
typedef struct {
  int32_t dim;
  int64_t n_elems;
  int64_t n_sides;
  int32_t elem_nv;
  const int64_t* side_elem_map;   /* [n_sides, 2]                          */
  const double* normal_areas;     /* [n_sides, dim]                        */
  const double* dists;            /* [n_sides, dim]                        */
  const double* elem_volumes;     /* [n_elems]                             */
  const double* side_areas;       /* [n_sides]                             */
  const double* interp_weights;   /* [n_sides]                             */
  const double* gradient_weights; /* [n_elems, dim, elem_nv]               */
  const int64_t* elem_side_map;   /* [n_elems, elem_nv]                    */
  int64_t n_internal;
  const int64_t* internal;
  int64_t n_periodic;
  const int64_t* periodic_sides;
  const double* periodic_jump;
  int64_t n_mixed;
  const int64_t* mixed_sides;
  const double* mixed_value;
  const double* mixed_conductance;
  int32_t contact_kind;           /* OBTE_CONTACT_NONE / PERIODIC / MIXED  */
  int64_t n_contact;
  const int64_t* contact_sides;
  double contact_alpha;           /* jump (periodic) or value (mixed)       */
  double contact_conductance;     /* mixed contact only                     */
  double normalization;
  const double* kappa;            /* [dim, dim] thermal conductivity        */
  const double* heat_source;      /* [n_elems] or NULL (W/m^3, x1e-18)       */
  int32_t pin_elem;               /* element pinned to 0 without mixed BCs (10) */
} obte_fourier_problem;

typedef struct {
  int32_t max_iter;               /* fourier_max_iter (40)                 */
  double rtol;                    /* fourier_rtol (1e-8)                   */
  double cg_rtol;                 /* inner CG tolerance                    */
  int32_t cg_max_iter;
} obte_fourier_opts;

typedef struct {
  double kappa;                   /* diffusive kappa (the value the reference prints) */
  int32_t n_iter;                 /* deferred-correction iterations        */
  int32_t n_cg;                   /* total CG iterations                   */
} obte_fourier_info;

obte_status obte_fourier_plan_create(obte_context ctx, const obte_fourier_problem* prob,
                                     obte_fourier_plan* out);
obte_status obte_fourier_plan_destroy(obte_fourier_plan plan);
/*   T device [n_elems] Temperature_Fourier;  J device [n_elems, dim] Flux_Fourier / 1e9 */
obte_status obte_fourier_solve(obte_fourier_plan plan, const obte_fourier_opts* opts, double* T,
                               double* J, obte_fourier_info* info);

#ifdef __cplusplus
}
#endif
#endif /* OBTE_H */
