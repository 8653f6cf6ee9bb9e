/*
 * ns3d_capi.h -- C-ABI of the NS3D steady staggered-grid Navier-Stokes
 * permeability solver (GB300 / sm_103a implementation).
 *
 * The reference solver (jerome-lux/NS3D) has no plugin API: its seam is the
 * C++ class NavierStokesBase (src/NSBase.h:63-594) driven by the four
 * XSOLVER::Solve(NavierStokesBase&) drivers and selected in main
 * (src/navierstokes3D.cxx:516-542).  Every entry point below replaces one
 * piece of that surface; the reference interface it stands for is cited on
 * each declaration.
 *
 * Conventions
 *  - Plain C types only; the caller owns every host buffer, the library owns
 *    device memory.
 *  - Every function returns an int status: NS3D_OK (0) or a negative API
 *    error.  Linear-solver outcomes use the numeric values of Eigen's
 *    ComputationInfo, which the reference prints as "(status N)" in its INFO
 *    log: Success 0, NumericalIssue 1, NoConvergence 2, InvalidInput 3.
 *  - No C++ exception crosses the ABI.  ns3d_last_error() returns the text of
 *    the last error raised on the calling thread.
 *  - A handle is used by one host thread at a time; separate handles may run
 *    concurrently (each owns its own CUDA stream).
 *  - Index maps are int32 in C order (i = x outermost, k = z fastest), the
 *    layout of the reference's blitz::Array<int,3> (src/NSBase.h:90-93), in
 *    the rotated/padded frame in which the flow runs along x.
 *
 * The CPU oracle under oracle/ implements this same header, so the two
 * libraries can be swapped for A/B runs.
 */
#ifndef NS3D_CAPI_H
#define NS3D_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define NS3D_API __declspec(dllexport)
#else
#define NS3D_API __attribute__((visibility("default")))
#endif

#define NS3D_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum {
    NS3D_OK = 0,
    /* linear-solver statuses (Eigen ComputationInfo values) */
    NS3D_SUCCESS = 0,
    NS3D_NUMERICAL_ISSUE = 1,
    NS3D_NO_CONVERGENCE = 2,
    NS3D_INVALID_INPUT = 3,
    /* API errors */
    NS3D_ERR_ARG = -1,         /* bad argument (NULL pointer, bad size, bad key value) */
    NS3D_ERR_OOM = -2,         /* device or host allocation failed */
    NS3D_ERR_CUDA = -3,        /* a CUDA call failed */
    NS3D_ERR_IO = -4,          /* file could not be opened / read / written */
    NS3D_ERR_PARSE = -5,       /* malformed ini or .vti content */
    NS3D_ERR_STATE = -6,       /* call out of order (e.g. fields before open) */
    NS3D_ERR_TIMEOUT = -7,     /* a bounded device wait ran out */
    NS3D_ERR_UNSUPPORTED = -8  /* feature not available in this build */
};

/* outer-loop algorithm, src/navierstokes3D.cxx:522-542 */
enum { NS3D_SIMPLEC = 0, NS3D_SIMPLER = 1, NS3D_SIMPLERR = 2, NS3D_IDEAL = 3 };

/* arithmetic of the inner solves */
/* NS3D_MIXED_MG: as NS3D_MIXED, with an aggregation multilevel preconditioner
 * (instead of Jacobi) in the FP32 pressure(-correction) solves */
enum { NS3D_FP64 = 0, NS3D_MIXED = 1, NS3D_MIXED_MG = 2 };

/* systems addressed by the step-level entry points */
enum { NS3D_SYS_U = 0, NS3D_SYS_V = 1, NS3D_SYS_W = 2, NS3D_SYS_P = 3 };

/*
 * Solver parameters: the ini keys of the reference (InputParams,
 * src/navierstokes3D.cxx:162-201), same names, meaning and defaults.
 * method/precision are integers (see the enums above).
 */
typedef struct ns3d_params {
    double dx, dy, dz;             /* grid spacing (m); dy,dz <= 0 mean "same as dx" */
    double mu, rho;                /* viscosity (Pa.s), density (kg/m^3) */
    double p0, gradp;              /* inlet pressure (Pa), imposed gradient (Pa/m) */
    double alpha, beta;            /* velocity / pressure relaxation */
    double vsolvertol, psolvertol, pcsolvertol;
    double simpletol, deltaRMR;
    int32_t maxitsolver, maxitSIMPLE, N1, N2, save_step;
    int32_t porevalue, direction, border;
    int32_t method, precision;
} ns3d_params;

/* grid and system sizes after rotation and border padding */
typedef struct ns3d_sizes {
    int32_t nx, ny, nz;
    int32_t np, nu, nv, nw;
    int32_t reserved;
} ns3d_sizes;

/* diagnostics of the last outer iteration and of the whole solve */
typedef struct ns3d_result {
    double K, Q, v_moy, RMR;
    double normdiv, reldiv, velocityNorm, maxdiv, MaxDeltaV;
    double p_inlet, p_outlet, p0, p1;
    double alpha, beta;
    double pcmax, pcmin, pcnorm;
    double seconds;                /* wall time of ns3d_solve */
    int32_t iterations;            /* loop index at exit ("terminated in N iteration") */
    int32_t converged;             /* CheckConvergence returned true */
    int32_t it_u, it_v, it_w, it_p;/* iterations() of the last u/v/w/p solve */
    int64_t krylov_iterations;     /* BiCGSTAB iterations summed over every solve */
    int64_t krylov_rows;           /* sum over solves of iterations x rows */
} ns3d_result;

/* outcome of one BiCGSTAB solve (Eigen iterations()/error()/info()) */
typedef struct ns3d_solve_info {
    int32_t iterations;
    int32_t info;
    double error;
} ns3d_solve_info;

typedef struct ns3d_handle ns3d_handle;

/* ---- library ----------------------------------------------------------- */
NS3D_API int ns3d_abi_version(void);
/* "gb300" for the CUDA library, "oracle" for the CPU restatement */
NS3D_API const char *ns3d_backend_name(void);
NS3D_API const char *ns3d_last_error(void);

/* Fill *p with the reference defaults, src/navierstokes3D.cxx:162-201. */
NS3D_API void ns3d_params_default(ns3d_params *p);

/* ---- geometry ---------------------------------------------------------- */
/*
 * Build a solver instance from a raw voxel image.
 * raw: nx*ny*nz bytes in VTK order (x fastest), as read from the .vti file
 *      (readvtkfile_uint8, src/vtkio.cxx:96-150): a voxel equal to
 *      params->porevalue is fluid.  Host memory, or device memory of the
 *      current device (the copy direction follows the pointer).
 * A parameter that is NaN or infinite returns NS3D_ERR_ARG before any device
 * work (the reference would carry it into every field).
 * The image is binarized, rotated so the flow runs along x
 * (NavierStokesBase::Rotation, src/NSBase.cxx:2451-2492), padded along x
 * (AddBorder, src/NSBase.cxx:2425-2448) and indexed
 * (InitIndexArrays, src/NSBase.cxx:2495-2573); p1 and the relaxation
 * constants are set as in the constructor (src/NSBase.cxx:155-179).
 * Replaces NavierStokesBase::NavierStokesBase (src/NSBase.cxx:50-194).
 */
NS3D_API int ns3d_open(const ns3d_params *params, const uint8_t *raw,
                       int32_t nx, int32_t ny, int32_t nz, ns3d_handle **out);

/* Sizes after rotation/padding and the counts np/nu/nv/nw
 * (NavierStokesBase members nx..nw, src/NSBase.h:77). */
NS3D_API int ns3d_get_sizes(const ns3d_handle *h, ns3d_sizes *s);

/* Copy the index maps (pindex, uindex, vindex, windex; src/NSBase.h:90-93).
 * Shapes: p,v,w nx*ny*nz; u (nx+1)*ny*nz.  Any pointer may be NULL. */
NS3D_API int ns3d_get_index_arrays(ns3d_handle *h, int32_t *pindex, int32_t *uindex,
                                   int32_t *vindex, int32_t *windex);

/* ---- fields ------------------------------------------------------------ */
/*
 * Initial fields, image-shaped in the rotated frame (p: nx*ny*nz,
 * u: (nx+1)*ny*nz, v,w: nx*ny*nz).  NULL keeps the default: the linear
 * pressure profile p0 + (p1-p0)(i+1)/nx (Initpvector, src/NSBase.cxx:2645-2690)
 * and zero velocity (InitVelocity, src/NSBase.cxx:2575-2642).  A NaN or an
 * infinity anywhere in a given array returns NS3D_ERR_ARG and leaves the
 * fields unchanged.
 */
NS3D_API int ns3d_set_initial_fields(ns3d_handle *h, const double *p_img, const double *u_img,
                                     const double *v_img, const double *w_img);

/* Compacted fields (lengths np, nu, nv, nw).  Any pointer may be NULL.
 * ns3d_set_fields rejects non-finite values like ns3d_set_initial_fields. */
NS3D_API int ns3d_get_fields(ns3d_handle *h, double *p, double *u, double *v, double *w);
NS3D_API int ns3d_set_fields(ns3d_handle *h, const double *p, const double *u,
                             const double *v, const double *w);

/*
 * Image-shaped fields as written by FieldsToImage (src/NSBase.cxx:330-476):
 * p, v, w: nx*ny*nz; u: (nx+1)*ny*nz; vavg: 3*nx*ny*nz interleaved
 * (face-averaged cell velocity).  Zeros where no node exists.  C order.
 */
NS3D_API int ns3d_get_field_images(ns3d_handle *h, double *p_img, double *u_img, double *v_img,
                                   double *w_img, double *vavg_img);

/* ---- logs and outputs -------------------------------------------------- */
/*
 * Write the INFO / RES logs (INFO-<dir>-<stem>.log, RES-<dir>-<stem>.csv,
 * src/NSBase.cxx:107-123) and, for the CUDA library, the field snapshots
 * and final .vti files (<stem>-SAVE-k.vti, P-/V-/Vx-/Vy-/Vz-<dir>-<stem>.vti)
 * into directory `dir`.  dir == NULL disables all file output.
 * write_fields = 0 keeps the logs but skips the .vti files.
 */
NS3D_API int ns3d_set_output(ns3d_handle *h, const char *dir, const char *stem,
                             int32_t write_fields);

/* ---- solve ------------------------------------------------------------- */
/*
 * Run the outer loop selected by params->method (SIMPLECSOLVER::Solve
 * src/SIMPLEC.cxx:73-232, SIMPLERSOLVER::Solve src/SIMPLER.cxx:75-270,
 * SIMPLERRSOLVER::Solve src/SIMPLERR.cxx:75-280, IDEALSOLVER::Solve
 * src/IDEAL.cxx:75-281) from the current initial fields.
 */
NS3D_API int ns3d_solve(ns3d_handle *h);
/*
 * Pressure-drop sweep on one image (no counterpart in the reference, which
 * solves one gradp per run; the Forchheimer analysis described in
 * doc/NS3D_methods.tex needs several): for each gradp[i] the handle's p0/p1
 * are re-derived (same rule as ns3d_open), the solve runs, and results[i]
 * receives its result.  Geometry, index arrays and systems are built once.
 * warm_start = 0: every solve starts from the default fields, so results[i]
 * equals ns3d_open + ns3d_solve with that gradp; warm_start = 1: solve i > 0
 * starts from solve i-1's fields scaled by gradp[i]/gradp[i-1] (exact for
 * Stokes flow).  The fields of the last solve stay in the handle.
 */
NS3D_API int ns3d_solve_sweep(ns3d_handle *h, const double *gradp, int32_t n, int32_t warm_start,
                              ns3d_result *results);
NS3D_API int ns3d_get_result(const ns3d_handle *h, ns3d_result *r);

/* ---- step-level entry points (one reference method each) --------------- */
/* AssembleAllMomentum on the current u,v,w (src/NSBase.cxx:853-884). */
NS3D_API int ns3d_assemble_momentum(ns3d_handle *h);
/* AssemblePressureCorrectionSIMPLEC (simplec=1, src/NSBase.cxx:612-732) or
 * ...SIMPLE (simplec=0, src/NSBase.cxx:734-851) on the current fields. */
NS3D_API int ns3d_assemble_pressure_correction(ns3d_handle *h, int32_t simplec);
/* Compute_{u,v,w}_hat (src/NSBase.cxx:1548-1755) with uc = u_old = current
 * velocity, then AssemblePressure (src/NSBase.cxx:478-610). */
NS3D_API int ns3d_assemble_pressure(ns3d_handle *h, int32_t relax);
/*
 * Copy the last assembled system `sys` (NS3D_SYS_*): coef is 7*n doubles,
 * slot-major [P,W,E,S,N,B,T][n] (missing entries are 0); nbr is 6*n int32
 * [W,E,S,N,B,T][n] (-1 = no entry); rhs n doubles; rowsum n doubles
 * (uA.row(r).sum(), momentum systems only).  Any pointer may be NULL.
 */
NS3D_API int ns3d_get_system(ns3d_handle *h, int32_t sys, double *coef, int32_t *nbr,
                             double *rhs, double *rowsum);
/*
 * BiCGSTAB with Jacobi preconditioning on the assembled system `sys`
 * (Eigen::BiCGSTAB::solveWithGuess as used at src/NSBase.cxx:1799,2343):
 * x holds the guess on entry and the solution on exit; rhs NULL uses the
 * system's assembled right-hand side.
 */
NS3D_API int ns3d_solve_system(ns3d_handle *h, int32_t sys, const double *rhs, double *x,
                               double tol, int32_t maxit, ns3d_solve_info *info);

NS3D_API int ns3d_close(ns3d_handle *h);

/* ---- measurement (no counterpart in the reference, which only times whole
 * solves with time(0), src/SIMPLEC.cxx:59,228-231) -------------------------- */
/* per-kernel device time of the pressure(-correction) BiCGSTAB kernels,
 * collected with CUDA events on the solver's stream while enabled */
typedef struct ns3d_profile {
    /* index 0-4: the phases of a BiCGSTAB iteration inside the loop kernel
     * (K1 p-update, K2 SpMV+dot, K3 s-update, K4 SpMV+dots, K5 x/r-update):
     * launches = iterations, ms = time between the grid barriers that end the
     * phases (global timer of block 0).  index 5: launches of the loop kernel,
     * ms by CUDA events.  rows: row-iterations of active systems. */
    int64_t launches[6];
    double ms[6];
    int64_t rows[6];
    int64_t total_launches;   /* kernels the library launched since profiling was enabled on this handle */
} ns3d_profile;
NS3D_API int ns3d_set_profiling(ns3d_handle *h, int32_t enable);
NS3D_API int ns3d_get_profile(ns3d_handle *h, ns3d_profile *out);
/* kernels this library launched in the process so far (every handle,
 * server and batch call) */
NS3D_API int64_t ns3d_kernel_launches(void);
/* pressure(-correction) solves of the handle's last solve that ran in mixed
 * precision, ended without success and were redone in FP64 (the precision
 * then stays FP64 for that solve's later pressure systems); 0 for FP64
 * handles, -1 for a NULL handle */
NS3D_API int32_t ns3d_mixed_fallbacks(const ns3d_handle *h);

/*
 * BiCGSTAB that allocates nothing.  No counterpart in the reference: it
 * exists for callers that cannot call cudaMalloc -- hosts running inside
 * another framework's memory pool or reserving all device memory at start-up,
 * and hosts that forbid allocation after initialisation.  The caller passes a
 * system already in device memory (coef 7*npad doubles slot-major
 * [P,W,E,S,N,B,T], nbr 6*npad int32 [W,E,S,N,B,T], -1 = no entry, npad a
 * multiple of 1024 and >= n), the right-hand side and the guess/solution x
 * (npad doubles each) and a CUDA stream (NULL = default stream).  Work vectors
 * live in a fixed device array inside the library: at most 65536 rows
 * (larger n returns NS3D_ERR_ARG); the array (about 4.5 MiB) is held until
 * exit.  CUDA loads a library's device code lazily by default, so the array
 * (and the kernels' code) are placed on a device by the first call on that
 * device, which also looks up the array's device address
 * (cudaGetSymbolAddress): make that first call before the host reserves the
 * rest of the device's memory and before any stream capture.  All calls
 * share the array: calls that overlap on the GPU race and must be serialized
 * by the caller.  Same arithmetic and results as ns3d_solve_system.  Error
 * text: ns3d_noalloc_last_error() (the text of this thread's last failed
 * call; a successful call clears it).
 */
NS3D_API int ns3d_bicgstab_noalloc(const double *coef, const int32_t *nbr, const double *rhs, double *x, int32_t n,
                                   int32_t npad, double tol, int32_t maxit, void *stream, ns3d_solve_info *info);
NS3D_API const char *ns3d_noalloc_last_error(void);

/* ---- synthetic images on the device (no counterpart in the reference, which
 * reads its geometry from .vti files, src/vtkio.cxx:96-150) ---------------- */
/*
 * Seeded porous image, nx*ny*nz uint8 in VTK order (x fastest; 1 = solid),
 * written to `raw` (host, may be NULL).  kind 0: overlapping balls of integer
 * radius with integer centres uniform in the box; kind 1: isotropic straight
 * fibres (unions of balls of that radius centred at rint(p + t d), t = -L,
 * -L+1, ... < L, L = box diagonal).  Primitives (from a splitmix64 stream of
 * `seed`) are added in order until the solid fraction reaches 1 - porosity.
 * *achieved = the resulting porosity; *nprims = primitives used; prims (may
 * be NULL) receives up to max_prims of them, 6 doubles each (centre or point,
 * then the unit direction of a fibre, zeros for a ball).
 */
NS3D_API int ns3d_generate_image(int32_t kind, int32_t nx, int32_t ny, int32_t nz, int32_t radius, double porosity,
                                 uint64_t seed, uint8_t *raw, double *achieved, double *prims, int32_t max_prims,
                                 int32_t *nprims);

/* ---- many solves on one GPU (no counterpart in the reference, which runs
 * one image per process, src/navierstokes3D.cxx:516-542) ------------------- */
/*
 * Batch: solve njobs independent images concurrently, at most max_concurrent
 * at a time, each on its own solver instance and CUDA stream.  raws[i] is the
 * i-th raw image (VTK order), dims[3i..3i+2] its size.  results[i] and
 * status[i] (may be NULL) receive each outcome.  Returns the worst status.
 */
NS3D_API int ns3d_batch_solve(const ns3d_params *params, const uint8_t *const *raws, const int32_t *dims,
                              int32_t njobs, int32_t max_concurrent, ns3d_result *results, int32_t *status);

/*
 * Server with continuous batching: requests are queued by ns3d_server_submit
 * (the image is copied), admitted as soon as fewer than max_active solves run
 * and the device has room for the request's estimated footprint
 * (hbm_budget_bytes = 0: the free memory the device reports), solved on their
 * own stream with their state resident in HBM until convergence, and
 * retired; the next requests are admitted as memory frees up.
 */
typedef struct ns3d_server ns3d_server;
typedef struct ns3d_server_stats {
    int64_t completed, failed, queued;
    int32_t active, peak_active;
    double p50_latency_s, p99_latency_s, mean_latency_s;
    double solves_per_s;  /* completed / (last completion - first submission) */
} ns3d_server_stats;
NS3D_API int ns3d_server_start(int32_t max_active, size_t hbm_budget_bytes, ns3d_server **out);
/* keep_fields != 0 keeps the compacted fields for ns3d_server_fields */
NS3D_API int ns3d_server_submit(ns3d_server *s, const ns3d_params *p, const uint8_t *raw, int32_t nx, int32_t ny,
                                int32_t nz, int32_t keep_fields, int64_t *ticket);
/* The same without copying the image: raw (host memory, or device memory of
 * the server's device -- an image generated or staged there) must stay valid
 * and unchanged until the request has finished or failed. */
NS3D_API int ns3d_server_submit_resident(ns3d_server *s, const ns3d_params *p, const uint8_t *raw, int32_t nx,
                                         int32_t ny, int32_t nz, int32_t keep_fields, int64_t *ticket);
/* state: 0 queued, 1 running, 2 done, 3 failed (the return value is the failure status) */
NS3D_API int ns3d_server_poll(ns3d_server *s, int64_t ticket, int32_t *state, ns3d_result *result);
NS3D_API int ns3d_server_wait(ns3d_server *s, int64_t ticket, ns3d_result *result, double *latency_s);
NS3D_API int ns3d_server_fields(ns3d_server *s, int64_t ticket, double *p, double *u, double *v, double *w);
NS3D_API int ns3d_server_get_stats(ns3d_server *s, ns3d_server_stats *out);
/* drops the requests not yet admitted (they end with NS3D_ERR_STATE) */
NS3D_API int ns3d_server_cancel_queued(ns3d_server *s, int64_t *cancelled);
/* finishes the queued and running requests, then frees the server */
NS3D_API int ns3d_server_stop(ns3d_server *s);

/*
 * Merged solve sets (no counterpart in the reference, which solves one image
 * per process with Eigen, src/NSBase.cxx:1799,1825,1852,2343,2393,2397).
 * Solver instances attached to one group pool their FP64 BiCGSTAB sets (the
 * three momentum components, the pressure(-correction) system; FP64, or FP32
 * inside FP64 defect correction) while they solve: one persistent
 * loop-kernel launch per round serves up to 64 FP64 (32 mixed) systems of
 * many images of different sizes, laid out as one ragged list of 1024-row
 * chunks.  Every system keeps its own Krylov scalars, reduction order and
 * preconditioner, so each result is bit-identical to the solve alone.
 * Attach with ns3d_set_group before ns3d_solve (NULL detaches); destroy a
 * group after every solve attached to it returned (ns3d_group_destroy
 * returns NS3D_ERR_STATE while one runs; a solve that starts while the
 * destroy runs fails with NS3D_ERR_STATE) and before any handle still
 * attached to it solves again.  The caller must make sure that no thread can
 * still reach the group (attach, solve) once ns3d_group_destroy returned OK:
 * the group's memory is freed.  The solves of a group must run on separate
 * host threads.
 */
typedef struct ns3d_group ns3d_group;
typedef struct ns3d_group_stats {
    int64_t launches;  /* merged solve sets run */
    int64_t requests;  /* member sets they served */
    int64_t systems;   /* linear systems they solved */
    int32_t max_systems, max_requests;  /* the largest merged set */
} ns3d_group_stats;
/* lanes (1-16): merged solves that may run at once, each for a cohort of
 * about members / lanes solves */
NS3D_API int ns3d_group_create(int32_t lanes, ns3d_group **out);
NS3D_API int ns3d_set_group(ns3d_handle *h, ns3d_group *g);
NS3D_API int ns3d_group_get_stats(ns3d_group *g, ns3d_group_stats *out);
NS3D_API int ns3d_group_destroy(ns3d_group *g);
/* lanes > 0: every request of the server solves in one group of that many
 * lanes; 0: no merging (before the first submit) */
NS3D_API int ns3d_server_set_merging(ns3d_server *s, int32_t lanes);
NS3D_API int ns3d_server_group_stats(ns3d_server *s, ns3d_group_stats *out);
/*
 * Lockstep solves (no counterpart in the reference, which solves one image
 * per process): the solves of n opened handles, any mix of the four methods
 * (SIMPLECSOLVER::Solve, src/SIMPLEC.cxx:73-232; SIMPLERSOLVER::Solve,
 * src/SIMPLER.cxx:75-270; SIMPLERRSOLVER::Solve, src/SIMPLERR.cxx:75-280;
 * IDEALSOLVER::Solve, src/IDEAL.cxx:75-281), driven together by the calling
 * thread.  Every image takes exactly its own steps -- result, fields and
 * logs are bit-identical to ns3d_solve of that handle -- but each stage of
 * an outer iteration runs for all images at once: their kernels on one
 * stream, each BiCGSTAB step as merged sets (one persistent launch per round
 * over the ragged chunk lists of all images, by each image's precision), one
 * host wait per read-back for all.  status[i] (may be NULL) receives each
 * outcome.  A handle attached to a solve group (ns3d_set_group) takes part
 * like any other: its BiCGSTAB steps join the lockstep call's merged sets,
 * not the group's.  The batch form opens, solves and closes n images (all of
 * them resident at once).
 */
NS3D_API int ns3d_solve_lockstep(ns3d_handle *const *hs, int32_t n, int32_t *status);
NS3D_API int ns3d_batch_solve_lockstep(const ns3d_params *params, const uint8_t *const *raws, const int32_t *dims,
                                       int32_t n, ns3d_result *results, int32_t *status);

/*
 * Autotuner of merged solve sets (no counterpart in the reference).  The
 * persistent loop kernel of a merged set may run on any number of blocks
 * without changing a bit of the results (fixed-order reductions); the
 * library times each candidate grid (the base grid / 1, 2, 4, 8) on three
 * live launches per class of set (solver kind, size, lanes) and then keeps
 * the fastest per row-iteration.  mode 0: off (base grid), 1: on (default),
 * 2: on with the measurements forgotten.  The table (one line per class;
 * `cap` bytes with the terminating zero) returns its full length.
 */
NS3D_API int ns3d_autotune_enable(int32_t mode);
NS3D_API int ns3d_autotune_table(char *buf, int32_t cap);

/*
 * Testing aid for the failure path of the persistent solver kernels (no
 * counterpart in the reference, which has no device code).  Their grid-wide
 * barriers wait a bounded time: after the limit a kernel sets an error flag,
 * stops, and the call that launched it returns NS3D_ERR_TIMEOUT with the
 * context intact.  While extra_arrivals > 0, every barrier of every loop-kernel
 * launch in the process waits for that many arrivals beyond the grid's own,
 * which never come, and gives up after limit_s seconds (> 0, at most 10), so
 * a test can watch that path end without a fault.  extra_arrivals = 0
 * restores normal launches.  Not for use while other solves run.
 */
NS3D_API int ns3d_debug_barrier_timeout(int32_t extra_arrivals, double limit_s);
/* ns3d_batch_solve with the solves merged in a group of `lanes` lanes;
 * stats (may be NULL) of the group */
NS3D_API int ns3d_batch_solve_merged(const ns3d_params *params, const uint8_t *const *raws, const int32_t *dims,
                                     int32_t njobs, int32_t max_concurrent, int32_t lanes, ns3d_result *results,
                                     int32_t *status, ns3d_group_stats *stats);

/* ---- host utilities (CUDA library only; no device work) ----------------- */
/*
 * Parse an ini file like ReadInput (src/navierstokes3D.cxx:266-463): same
 * keys, defaults, validation and messages (written to stderr).  The file
 * keys (input, pressurefield, vxfield, vyfield, vzfield) are copied into the
 * caller's buffers of `cap` bytes each (any may be NULL).  One key is added
 * to the reference's set: precision = FP64 | MIXED.
 * Returns NS3D_OK, NS3D_ERR_IO (cannot open) or NS3D_ERR_PARSE (fatal error).
 */
NS3D_API int ns3d_ini_read(const char *path, ns3d_params *p, char *input, char *pressurefield, char *vxfield,
                           char *vyfield, char *vzfield, size_t cap);
/*
 * Read a .vti (VTK XML ImageData, appended/inline, raw/base64, zlib or not)
 * or legacy .vtk STRUCTURED_POINTS file (readvtkfile_uint8 /
 * readvtkfile_double, src/vtkio.cxx:38-150).  dims receives nx, ny, nz and
 * ncomp the component count; values are returned in file order (x fastest).
 * With buf == NULL only the sizes are returned.  cap is the buffer length in
 * elements.
 */
NS3D_API int ns3d_vti_read_u8(const char *path, uint8_t *buf, size_t cap, int32_t dims[3]);
NS3D_API int ns3d_vti_read_f64(const char *path, double *buf, size_t cap, int32_t dims[3], int32_t *ncomp);
/* Write nx*ny*nz*ncomp doubles given in C order (x slowest) as a Float64
 * zlib-compressed appended .vti (writeScalarImage / writeVectorImage,
 * src/vtkio.cxx:161-246). */
NS3D_API int ns3d_vti_write_f64(const char *path, const double *data, int32_t nx, int32_t ny, int32_t nz,
                                int32_t ncomp);
/* Write a binary uint8 image given in file order (x fastest)
 * (writeBinaryImage, src/vtkio.cxx:254-291). */
NS3D_API int ns3d_vti_write_u8(const char *path, const uint8_t *data, int32_t nx, int32_t ny, int32_t nz);
/*
 * The NS3D program: read the ini, the image and the restart fields, solve,
 * write INFO/RES logs and the .vti fields into out_dir (NULL = current
 * directory) -- main, src/navierstokes3D.cxx:480-545.  If result is not NULL
 * it receives the final diagnostics.
 */
NS3D_API int ns3d_run_ini(const char *ini_path, const char *out_dir, ns3d_result *result);

#ifdef __cplusplus
}
#endif

#endif /* NS3D_CAPI_H */
