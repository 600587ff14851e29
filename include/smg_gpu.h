/*
 * smg_gpu.h — C ABI of the GB300 (sm_103a) Wilson-clover Dirac operator and
 * multigrid solve path for the 2D U(1) lattice Schwinger model.
 *
 * Every entry point takes plain pointers and sizes; no C++ or torch types
 * cross this boundary.  Objects are opaque handles with explicit
 * create/destroy.  Device memory belongs to the library; host arrays passed
 * in are read (or written) before the call returns and are never retained.
 *
 * Host array conventions (identical to the reference's `Vec`/`GaugeField`):
 *   - complex numbers are interleaved (re, im) doubles;
 *   - a spinor is `v[2*s + spin]` with lexicographic site s = x + L*y
 *     (reference src/types.h:8, src/lattice.h:19), i.e. 2*V complex = 4*V
 *     doubles; a multi-RHS field is nrhs such spinors back to back;
 *   - gauge links are `U[mu][s]`, mu = 0 (x) then 1 (y)
 *     (reference src/gauge.h:12), i.e. 2*V complex = 4*V doubles;
 *   - a force / momentum field is `F[mu][s]` real, 2*V doubles
 *     (reference src/hmc.h:34).
 *
 * Each function returns an smg_status; SMG_OK is 0.  The reference signals
 * failure through asserts, std::cerr warnings and early loop exits
 * (reference src/prolongator.h:38, src/solvers.cpp:765, src/coarse_op.h:533);
 * here every such condition maps to a status code, and
 * smg_last_error() gives the message of the last failure in a context.
 *
 * Threading: one smg_context per host thread (or per CUDA stream); objects of
 * distinct contexts may be used concurrently.  All work of a context is
 * enqueued on that context's stream; calls that return host data synchronise
 * that stream.
 */
#ifndef SMG_GPU_H
#define SMG_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SMG_API __attribute__((visibility("default")))

typedef enum {
    SMG_OK = 0,
    SMG_NOT_CONVERGED = 1,  /* iteration limit reached above tolerance      */
    SMG_BREAKDOWN = 2,      /* zero / tiny denominator in a Krylov step      */
    SMG_NONFINITE = 3,      /* NaN or Inf met in a residual or input         */
    SMG_BAD_ARG = 4,        /* invalid size, null pointer or mismatch        */
    SMG_DEVICE_ERROR = 5,   /* a CUDA call failed                            */
    SMG_TIMEOUT = 6,        /* a bounded device-side wait ran out            */
    SMG_NO_MEMORY = 7,      /* device allocation failed                      */
    SMG_UNSUPPORTED = 8,    /* configuration not built in this library       */
    SMG_IO_ERROR = 9        /* a file could not be opened, read or written   */
} smg_status;

typedef enum {
    SMG_F64 = 0,   /* complex128 storage and arithmetic                      */
    SMG_F32 = 1,   /* complex64 storage, FP32 arithmetic                     */
    SMG_F16 = 2    /* FP16 storage with one FP32 scale per site, FP32 math   */
} smg_precision;

/* Operators a Dirac handle can apply (reference src/dirac.h:115-152). */
typedef enum {
    SMG_OP_D = 0,       /* DiracOp::apply        dirac.h:115 */
    SMG_OP_DDAG = 1,    /* DiracOp::apply_dag    dirac.h:120 */
    SMG_OP_DDAGD = 2,   /* DiracOp::apply_DdagD  dirac.h:136 */
    SMG_OP_G5D = 3      /* DiracOp::apply_g5D    dirac.h:145 */
} smg_operator;

/* Even-odd (Schur complement) operators (reference EvenOddDiracOp,
 * src/dirac.h:190-553).  They act on full fields whose odd half holds the
 * reference's odd-site half vector (and even half its even-site vector):
 * half-vector index i = eo_index[s] = (x + L y) / 2 is the site order within
 * a parity half of a field. */
typedef enum {
    SMG_EO_SCHUR = 0,           /* M = D_oo - D_oe D_ee^-1 D_eo   apply_schur          dirac.h:425 */
    SMG_EO_SCHUR_DAG = 1,       /* M^dag = g5 M(-mu) g5           apply_schur_dag      dirac.h:430 */
    SMG_EO_SCHUR_DAG_SCHUR = 2, /* M^dag M                        apply_schur_dag_schur dirac.h:441 */
    SMG_EO_HOP_EO = 3,          /* even half -> odd half hopping  apply_eo             dirac.h:252 */
    SMG_EO_HOP_OE = 4           /* odd half -> even half hopping  apply_oe             dirac.h:257 */
} smg_eo_operator;

typedef struct smg_context smg_context;
typedef struct smg_gauge smg_gauge;
typedef struct smg_dirac smg_dirac;
typedef struct smg_field smg_field;
typedef struct smg_mg smg_mg;
typedef struct smg_batch smg_batch;
typedef struct smg_prolongator smg_prolongator;
typedef struct smg_coarse_op smg_coarse_op;

/* Result of a Krylov solve; mirrors CGResult / FCGResult
 * (reference src/solvers.h:25-35).  final_residual is the solver's own
 * (recursive) relative residual as the reference reports it; true_residual
 * is ||b - A x|| / ||b|| recomputed in FP64 after the solve.  For a
 * multi-RHS solve the fields hold the worst right-hand side. */
typedef struct {
    int iterations;
    double final_residual;
    double true_residual;
    int operator_applications;  /* fine-grid A applications (D^dag D) */
} smg_solve_result;

/* ---------------------------------------------------------------- context */

/* Creates a context on CUDA device `device`, enqueuing all work on `stream`
 * (a cudaStream_t; NULL = the library creates its own non-blocking stream).
 * No reference counterpart: the reference is a single-threaded CPU library
 * with process globals (reference src/linalg.cpp:5-6). */
SMG_API smg_status smg_context_create(int device, void* stream, smg_context** out);
SMG_API smg_status smg_context_destroy(smg_context* ctx);
SMG_API smg_status smg_context_synchronize(smg_context* ctx);
SMG_API smg_status smg_context_set_stream(smg_context* ctx, void* stream);
SMG_API void* smg_context_stream(smg_context* ctx);
SMG_API const char* smg_last_error(smg_context* ctx);
SMG_API const char* smg_status_string(smg_status s);
/* Number of kernels this context has launched since creation (a counter the
 * benchmark reads to report launches inside a timed region). */
SMG_API uint64_t smg_context_kernel_launches(smg_context* ctx);
/* Library version string, e.g. "smg-gb300 0.1 sm_103a". */
SMG_API const char* smg_version(void);
/* Stream-ordered timing on the context's stream: smg_timer_begin records a
 * CUDA event, smg_timer_end records a second one, waits for it and returns
 * the elapsed device time in milliseconds.  No reference counterpart (the
 * reference times with std::chrono, e.g. src/mode_studies.cpp:1554). */
SMG_API smg_status smg_timer_begin(smg_context* ctx);
SMG_API smg_status smg_timer_end(smg_context* ctx, double* ms);

/* ------------------------------------------------------------ gauge field */

/* GaugeField (reference src/gauge.h:10-36).  L must be even and >= 4.
 * U is 2*V complex, U[mu][s]. */
SMG_API smg_status smg_gauge_create(smg_context* ctx, int L, const double* U, smg_gauge** out);
SMG_API smg_status smg_gauge_destroy(smg_gauge* g);
SMG_API smg_status smg_gauge_set(smg_gauge* g, const double* U);
SMG_API smg_status smg_gauge_get(smg_gauge* g, double* U);
SMG_API int smg_gauge_L(const smg_gauge* g);
/* GaugeField::avg_plaq (reference src/gauge.h:32-36). */
SMG_API smg_status smg_gauge_avg_plaq(smg_gauge* g, double* out);
/* gauge_action = -beta * sum_s Re P(s) (reference src/hmc_forces.cpp:80-86). */
SMG_API smg_status smg_gauge_action(smg_gauge* g, double beta, double* out);
/* gauge_force (reference src/hmc_forces.cpp:88-111): force is 2*V doubles. */
SMG_API smg_status smg_gauge_force(smg_gauge* g, double beta, double* force);

/* ---------------------------------------------------------- Dirac operator */

/* DiracOp(lat, gauge, mass, r, c_sw, mu_t) (reference src/dirac.h:17-22).
 * Computes the clover field F01 on the device when c_sw != 0
 * (reference src/dirac.h:26-52).  The Dirac handle reads the gauge handle's
 * links at every apply; after smg_gauge_set call smg_dirac_refresh so the
 * clover term follows the new links. */
SMG_API smg_status smg_dirac_create(smg_gauge* g, double mass, double r, double c_sw,
                                    double mu_t, smg_dirac** out);
SMG_API smg_status smg_dirac_destroy(smg_dirac* d);
SMG_API smg_status smg_dirac_refresh(smg_dirac* d);
/* DiracOp::clover_field, V doubles (reference src/dirac.h:15). */
SMG_API smg_status smg_dirac_get_clover(smg_dirac* d, double* F01);
/* dst = op(src) for every right-hand side (reference src/dirac.h:115-152).
 * src and dst must have the same L, nrhs and precision and be distinct. */
SMG_API smg_status smg_dirac_apply(smg_dirac* d, smg_operator op, const smg_field* src,
                                   smg_field* dst);
/* DiracOp::apply_delta_D (reference src/dirac.h:154-174): dst = (D(e^{i dt pi} U)
 * - D(U)) src through the hopping terms (the reference leaves the clover term
 * out); pi is 2*V doubles [mu][s] on the host.  F64 fields. */
SMG_API smg_status smg_dirac_apply_delta(smg_dirac* d, const double* pi, double dt, const smg_field* src,
                                         smg_field* dst);

/* ---------------------------------------------------------- spinor fields */

/* A field holds nrhs spinors of an L x L lattice in the given precision.
 * Device layout is even-odd, site-major, right-hand side innermost. */
SMG_API smg_status smg_field_create(smg_context* ctx, int L, int nrhs, smg_precision prec,
                                    smg_field** out);
SMG_API smg_status smg_field_destroy(smg_field* f);
/* host: nrhs * 2V complex in the reference's Vec layout. */
SMG_API smg_status smg_field_upload(smg_field* f, const double* host);
SMG_API smg_status smg_field_download(const smg_field* f, double* host);
/* Same as upload/download but from/to page-locked host memory without an
 * intermediate staging copy; `host` must be pinned (cudaHostAlloc). */
SMG_API smg_status smg_field_upload_async(smg_field* f, const double* host);
SMG_API smg_status smg_field_download_async(const smg_field* f, double* host);
SMG_API smg_status smg_field_zero(smg_field* f);
/* dst = src with precision conversion (same L and nrhs). */
SMG_API smg_status smg_field_copy(const smg_field* src, smg_field* dst);
SMG_API int smg_field_nrhs(const smg_field* f);
SMG_API int smg_field_L(const smg_field* f);
SMG_API smg_precision smg_field_precision(const smg_field* f);
/* Raw device pointer and byte size of the field's storage. */
SMG_API void* smg_field_device_ptr(smg_field* f);
SMG_API size_t smg_field_bytes(const smg_field* f);

/* ------------------------------------------------------------------ BLAS-1 */

/* dot(a,b) = sum conj(a) b per right-hand side, out = nrhs complex
 * (reference src/linalg.cpp:8-18). Reductions accumulate in FP64. */
SMG_API smg_status smg_blas_dot(const smg_field* a, const smg_field* b, double* out);
/* norm(v) per right-hand side, out = nrhs doubles (reference src/linalg.cpp:20). */
SMG_API smg_status smg_blas_norm(const smg_field* a, double* out);
/* y += alpha x, alpha = nrhs complex (reference src/linalg.cpp:22-26). */
SMG_API smg_status smg_blas_axpy(const double* alpha, const smg_field* x, smg_field* y);
/* v *= alpha, alpha = nrhs complex (reference src/linalg.cpp:35-39). */
SMG_API smg_status smg_blas_scale(const double* alpha, smg_field* v);

/* Dot products that allocate nothing.  No counterpart in the reference: it
 * exists for callers that cannot call cudaMalloc when they need the result,
 * such as a framework that owns all device memory through its own pool, a
 * latency-critical loop that cannot afford an allocation, or a process under
 * a fixed device-memory budget.  a and b are device pointers to nrhs vectors
 * of n complex128 values each, stored one after another; out is a device
 * pointer that receives nrhs complex results sum_i conj(a_i) b_i as
 * interleaved (re, im) doubles.  Work is enqueued on `stream` (a cudaStream_t,
 * NULL = the legacy default stream) of the current device, and the call
 * returns without waiting for it.  Limit: nrhs <= 16 (larger values return
 * SMG_BAD_ARG); any n.  The scratch is a fixed 78,080-byte array that every
 * GPU loading this library keeps until the process exits; it is shared by all
 * calls and keeps the last call's contents, so calls whose kernels overlap on
 * the GPU (different streams, or different host threads on one device) race
 * and must be serialised by the caller.  The first call on each device looks
 * the array's device address up; make that first call before any stream
 * capture.  The address is kept for the life of the process: after
 * cudaDeviceReset (or anything else that re-creates the device's primary
 * context) it is stale, so do not call this function again in that process.
 * A launch error that the caller's own earlier work left pending is not
 * cleared: the call returns SMG_DEVICE_ERROR without launching. */
SMG_API smg_status smg_blas_dot_noalloc(const double* a, const double* b, int64_t n, int nrhs, double* out,
                                        void* stream);

/* ---------------------------------------------------------------- solvers */

/* cg_solve on A = D^dag D (reference src/solvers.cpp:16-78): unpreconditioned
 * CG from x = 0, stopping when the recursive ||r||/||b|| < tol.  Runs in the
 * precision of the fields (F64 or F32); every right-hand side is solved
 * independently and stops on its own. */
SMG_API smg_status smg_cg_solve(smg_dirac* d, const smg_field* rhs, smg_field* x,
                                int max_iter, double tol, smg_solve_result* res);
/* The same solve to a true FP64 residual below tol with FP32 CG inside FP64
 * defect correction: each outer step solves A e = r/||r|| with the FP32
 * operator and adds x += ||r|| e.  F64 fields only; iterations count the
 * FP32 CG iterations. */
SMG_API smg_status smg_cg_solve_mixed(smg_dirac* d, const smg_field* rhs, smg_field* x,
                                      int max_iter, double tol, smg_solve_result* res);

/* Preconditioned CG (the reference's cg_solve_core, src/solvers.cpp:16-72,
 * as cg_solve_precond / cg_solve_x0 / cg_solve_x0_precond, :80-96).  mg: one
 * MG cycle per iteration as the preconditioner (NULL: none); use_x0 != 0:
 * x holds the start vector on entry (else x = 0).  Complex alpha = <r,z>/<p,Ap>
 * and beta = <r',z'>/<r,z> per right-hand side; each stops on its own when
 * the recursive ||r||/||b|| < tol.  F64 or F32 fields. */
SMG_API smg_status smg_cg_solve_precond(smg_dirac* d, smg_mg* mg, const smg_field* rhs, smg_field* x,
                                        int use_x0, int max_iter, double tol, smg_solve_result* res);

/* mr_smooth (reference src/smoother.cpp:9-23): niter MR steps on A = D^dag D
 * from the x given on entry, omega = <Ar, r> / <Ar, Ar> per right-hand side. */
SMG_API smg_status smg_mr_smooth(smg_dirac* d, const smg_field* b, smg_field* x, int niter);
/* richardson_smooth_op on A = D^dag D (src/smoother.cpp:64-73): x += omega (b - A x),
 * niter steps from the x given on entry, omega > 0 fixed. */
SMG_API smg_status smg_richardson_smooth(smg_dirac* d, const smg_field* b, smg_field* x, int niter,
                                         double omega);
/* estimate_lambda_max of A = D^dag D (src/smoother.cpp:43-60): niter power
 * steps from random_vec(2V, std::mt19937(12345)); lambda = ||A v|| of the last. */
SMG_API smg_status smg_estimate_lambda_max(smg_dirac* d, int niter, double* lambda);

/* --------------------------------------------------------------- even-odd */

/* Applies an even-odd operator: Schur operators read the odd half of src and
 * write the odd half of dst; the hops read one half and write the other. */
SMG_API smg_status smg_eo_apply(smg_dirac* d, smg_eo_operator op, const smg_field* src, smg_field* dst);
/* EvenOddDiracOp::reconstruct (src/dirac.h:527-540): with x_o in the odd half
 * of x, writes x_e = D_ee^-1 (phi_e - D_oe x_o) into its even half; phi ==
 * NULL gives reconstruct_full (x_e = -D_ee^-1 D_oe x_o, :499-508). */
SMG_API smg_status smg_eo_reconstruct(smg_dirac* d, const smg_field* phi, smg_field* x);
/* EvenOddDiracOp::log_det_ee (src/dirac.h:511-521): Re log det D_ee. */
SMG_API smg_status smg_eo_logdet_ee(smg_dirac* d, double* logdet);
/* cg_solve on M^dag M over the odd halves (the e/o HMC solve,
 * src/hmc_trajectory.cpp:70-104): rhs and x are full fields of which the odd
 * halves are used; the even half of x is set to zero. */
SMG_API smg_status smg_eo_cg_solve(smg_dirac* d, const smg_field* rhs, smg_field* x, int max_iter, double tol,
                                   smg_solve_result* res);
/* eo_fermion_force (src/hmc_forces.cpp:812-867): F = -dS/dtheta for
 * S = phi_o^dag (M^dag M)^-1 phi_o - 2 log det D_ee at x_o = the odd half of
 * X (single-RHS F64); y_o = M x_o and the even-site reconstructions are
 * recomputed on the device.  force is 2*V doubles [mu][s]. */
SMG_API smg_status smg_eo_fermion_force(smg_dirac* d, const smg_field* X, double* force);

/* -------------------------------------------------------------- multigrid */

#define SMG_MAX_LEVELS 6

/* Parameters of an MG hierarchy for A = D^dag D (reference src/config.h:19-30,
 * src/multigrid.cpp:595-687).  Level 0 aggregates block[0][0] x block[0][1]
 * fine sites; level l >= 1 aggregates block[l][0] x block[l][1] sites of the
 * level-l coarse lattice.  The reference's linear blocking of 4k consecutive
 * coarse dofs (src/prolongator.h:149-228) is the aggregate 4 x 1 when the
 * coarse lattice width is a multiple of 4.  With chiral_split, each null
 * vector v gives the two block vectors of (1 +- sigma3) v / 2, so a level has
 * 2 * n_vec coarse dofs per site; without it, n_vec (the reference). */
typedef struct {
    int n_levels;                      /* 2 .. SMG_MAX_LEVELS              */
    int block[SMG_MAX_LEVELS - 1][2];  /* aggregate per level transition   */
    int n_vec[SMG_MAX_LEVELS - 1];     /* null vectors per transition      */
    int chiral_split;                  /* 0: reference; 1: split by sigma3 */
    int null_iters;                    /* inverse iterations (build_full_mg: 20) */
    int null_mr_steps;                 /* MR steps per inverse iteration (5)    */
    int pre_smooth, post_smooth;       /* MR steps per level (reference 3, 3)   */
    int w_cycle;                       /* second coarse visit at levels < last-1 */
    int coarse_max_iter;               /* coarsest CG (reference 200)           */
    double coarse_tol;                 /* coarsest CG (reference 1e-12)         */
    smg_precision precision;           /* F64, or F32 smoother and coarse levels */
    uint32_t seed;                     /* std::mt19937 seed of the start vectors */
    int tensor_cores;                  /* 1 (default): an F32 hierarchy applies its coarse operators
                                          with 16 dofs per site to multiples of 32 right-hand sides
                                          on the tensor cores (BF16 operands, FP32 accumulation);
                                          0: FP32 on the CUDA cores */
    int smoother_half;                 /* 1: an F32 hierarchy keeps the fine-level smoother's work
                                          vectors (residual, A r, D r) in FP16 with one FP32 scale
                                          per site, arithmetic in FP32 (power-of-two nrhs from 8
                                          to 32); 0 (default): FP32 */
    int coarse_half;                   /* 1: an F32 hierarchy keeps the coarse solves' work vectors
                                          in FP16 with FP32 scales (per coarse site and half of the
                                          32 right-hand sides): the coarsest-level CG's residual and
                                          search directions, and the MR residuals and A r of the
                                          intermediate levels (the tensor-core path: 16 dofs, 32
                                          right-hand sides); solutions, arithmetic and accumulation
                                          in FP32; 0 (default): FP32 */
} smg_mg_params;

/* Fills p with the reference's defaults: 2 levels, 4 x 4 blocks, 4 null
 * vectors, no chirality split, 20 inverse iterations of 5 MR steps, 3 + 3 MR
 * smoothing, W-cycle, coarsest CG 200 iterations to 1e-12, FP64
 * (reference src/config.h:19-30, src/mg_builder.cpp:18). */
SMG_API smg_status smg_mg_params_default(smg_mg_params* p);

/* build_mg_hierarchy / build_full_mg (reference src/multigrid.cpp:595-687,
 * src/mg_builder.cpp:3-31): near-null vectors by inverse iteration
 * (src/multigrid.cpp:435-484, 545-587), block-orthonormalised prolongators
 * (src/prolongator.h:111-141) and 9-point Galerkin coarse operators, built
 * directly from D P rather than by probing (src/coarse_op.h:241-279).
 * warm_start: NULL, or n_vec[0] level-0 start vectors (each 2V complex in the
 * reference layout) used instead of random draws, as build_mg_hierarchy's
 * warm_start argument.  Every coarse lattice must be at least 3 x 3. */
SMG_API smg_status smg_mg_create(smg_dirac* d, const smg_mg_params* p, const double* warm_start,
                                 smg_mg** out);
/* build_mg_hierarchy with the caller's generator (src/multigrid.cpp:595-687,
 * src/mg_builder.cpp:3-31): start_vecs[l], l < n_levels - 1, holds the
 * n_vec[l] start vectors of level l (random_vec draws, each nsites_l *
 * ndof_l complex: 2V at level 0) in the order the reference draws them from
 * its std::mt19937, so the hierarchy equals the reference's for the same
 * generator state; null_iters inverse iterations follow as in smg_mg_create. */
SMG_API smg_status smg_mg_create_from_starts(smg_dirac* d, const smg_mg_params* p, const double* const* start_vecs,
                                             smg_mg** out);
SMG_API smg_status smg_mg_destroy(smg_mg* mg);
/* ------------------------------------------------------ coarse deflation */

/* Outcome of the thick-restart Lanczos run of smg_mg_setup_deflation
 * (TRLMResult, reference src/eigensolver.h). */
typedef struct {
    int converged;
    int restarts;
    int iterations; /* Lanczos steps */
    int n_kr;       /* Krylov space size used */
} smg_deflation_info;

/* SparseCoarseOp::setup_deflation with the default TRLM solver (reference
 * src/coarse_op.cpp:10-54, trlm_eigensolver src/eigensolver_core.cpp:691):
 * the n_ev lowest eigenpairs of the level-1 operator A_c = P^dag D^dag D P,
 * held by the hierarchy.  n_kr <= 0 selects min(2 n_ev + 10, dim); the
 * reference's setup_sparse_coarse passes max_restarts = 100, tol = 1e-10.
 * With eigenpairs held and level 1 the coarsest level, the coarsest CG starts
 * from the deflated guess x0 = sum_i v_i (v_i^dag b) / lambda_i
 * (SparseCoarseOp::solve, src/coarse_op.h:492-547).  n_ev = 0 clears the
 * space.  Returns SMG_NOT_CONVERGED (pairs still stored) when Lanczos did not
 * converge within max_restarts. */
SMG_API smg_status smg_mg_setup_deflation(smg_mg* mg, int n_ev, int n_kr, int max_restarts, double tol,
                                          smg_deflation_info* info);
/* smg_mg_setup_deflation on the operator of coarse level `level` (1 = the
 * reference's choice).  With level the coarsest level, the coarsest CG of
 * every cycle starts from the deflated guess; the low-mode solution needs
 * level 1. */
SMG_API smg_status smg_mg_setup_deflation_level(smg_mg* mg, int level, int n_ev, int n_kr, int max_restarts,
                                                double tol, smg_deflation_info* info);
/* Replaces the eigenpairs (defl_vecs / defl_vals): n vectors of the level-1
 * dimension, interleaved complex128, in the reference's coarse layout
 * c[b * k + kv] with b the lexicographic coarse site. */
SMG_API smg_status smg_mg_set_deflation(smg_mg* mg, int n, const double* vals, const double* vecs);
/* Copies out the eigenpair count and (when the pointers are non-null) the
 * values and vectors in the layout of smg_mg_set_deflation. */
SMG_API smg_status smg_mg_get_deflation(smg_mg* mg, int* n, double* vals, double* vecs);
/* rr_evolve on the current level-1 operator (reference
 * src/eigen_evolve.cpp:48-105, as evolve_coarse_deflation applies it after
 * the coarse operator was rebuilt, src/hmc_multiscale.cpp:278-331 without
 * forecasting): Rayleigh-Ritz of the held vectors; max_residual (optional)
 * receives max_i ||A v_i - lambda_i v_i|| / ||A v_i||. */
SMG_API smg_status smg_mg_deflation_rr(smg_mg* mg, double* max_residual);
/* CoarseDeflState::lowmode_solution (reference src/hmc.h:312-323):
 * x = P sum_i v_i (v_i^dag P^dag phi) / lambda_i for single-RHS F64 fields
 * (terms with lambda_i <= 1e-14 skipped). */
SMG_API smg_status smg_mg_lowmode_solution(smg_mg* mg, const smg_field* phi, smg_field* x);

/* MGHierarchy::rebuild_deeper_levels with the level-0 Galerkin rebuild it
 * assumes (reference src/multigrid.cpp:158-193): after the gauge field of the
 * hierarchy's Dirac handle changed (smg_gauge_set + smg_dirac_refresh), every
 * coarse operator is recomputed from the existing prolongators; no new
 * near-null vectors are computed. */
SMG_API smg_status smg_mg_rebuild(smg_mg* mg);
/* Sizes of level `level` (0 = fine): lattice width/height in sites and dofs
 * per site. */
SMG_API smg_status smg_mg_level_dims(smg_mg* mg, int level, int* nx, int* ny, int* ndof);
/* MGHierarchy::null_vecs_l0: n_vec[0] vectors of 2V complex. */
SMG_API smg_status smg_mg_null_vectors(smg_mg* mg, double* out);
SMG_API smg_status smg_mg_n_null_vectors(smg_mg* mg, int* k);
/* Failure-path testing, no reference counterpart: the number of polls a
 * grid-barrier wait of the coarsest-level CG kernel makes before it gives up
 * (spins >= 0; 0 gives up at the first poll; < 0 restores the default of
 * about one second).  A wait that gives up ends the kernel and the next call
 * returns SMG_TIMEOUT (smg_mg_precondition and the solvers check the flag);
 * the hierarchy stays usable.  Drops the captured cycle graph. */
SMG_API smg_status smg_mg_set_wait_limit(smg_mg* mg, long long spins);
/* Block vectors of the prolongator from level `level` to level+1 in the
 * reference layout [block][k][local dof] (src/prolongator.h:23) where a local
 * dof of level 0 is 2*(lx + bx*ly) + spin and of level l >= 1 is
 * (lx + ax*ly) * ndof_l + j. */
SMG_API smg_status smg_mg_get_prolongator(smg_mg* mg, int level, double* block_vecs);
/* Coarse operator of level `level` >= 1 as SparseCoarseOp::link
 * (src/coarse_op.h:159-166): [site][dir][ki * k + kj] complex. */
SMG_API smg_status smg_mg_get_coarse_op(smg_mg* mg, int level, double* links);
/* x = M^-1 b, one MG cycle (MGHierarchy::precondition, src/multigrid.cpp:155;
 * mg_cycle, :43-102).  b and x are fine fields of the hierarchy's L.  The
 * cycle is replayed as a CUDA graph per (nrhs, precision); with the
 * environment variable SMG_CUDA_GRAPHS=0 at smg_mg_create it is launched
 * kernel by kernel instead. */
SMG_API smg_status smg_mg_precondition(smg_mg* mg, const smg_field* b, smg_field* x);
/* estimate_lambda_max (src/smoother.cpp:43-60) of the level-`level` operator
 * (0: D^dag D) in FP64 from random_vec(dim, std::mt19937(12345)). */
SMG_API smg_status smg_mg_estimate_lambda_max(smg_mg* mg, int level, int niter, double* lambda);
/* MGHierarchy::set_symmetric (src/multigrid.cpp:144-152): every level but the
 * coarsest smooths with Richardson at omega = damping / lambda_max (30 power
 * steps), which makes the cycle linear and Hermitian for CG; damping <= 0
 * returns to MR.  omega (optional) receives n_levels - 1 values. */
SMG_API smg_status smg_mg_set_symmetric(smg_mg* mg, double damping, double* omega);
/* Host-array versions of the transfer operators and the coarse operator at
 * level `level` (Prolongator::prolong / restrict_vec, src/prolongator.h:77-108;
 * SparseCoarseOp::apply_to, src/coarse_op.h:282-297).  Vectors use the
 * reference's dof order: fine 2*s + spin, coarse site * ndof + j. */
SMG_API smg_status smg_mg_prolong_host(smg_mg* mg, int level, const double* coarse, double* fine);
SMG_API smg_status smg_mg_restrict_host(smg_mg* mg, int level, const double* fine, double* coarse);
SMG_API smg_status smg_mg_coarse_apply_host(smg_mg* mg, int level, const double* in, double* out);
/* ----------------------------------- prolongator and sparse coarse operator */

/* Prolongator(lat, bx, by, k) + build_from_vectors (src/prolongator.h:14-142):
 * k null vectors (each 2V complex, reference layout) cut to bx x by blocks and
 * orthonormalised per block on the device.  L / bx and L / by >= 3. */
SMG_API smg_status smg_prolongator_create(smg_context* ctx, int L, int bx, int by, int k, const double* null_vecs,
                                          smg_prolongator** out);
SMG_API smg_status smg_prolongator_destroy(smg_prolongator* P);
/* Prolongator::block_vecs in the layout [block][k][2 * (lx + bx * ly) + spin]. */
SMG_API smg_status smg_prolongator_get_block_vecs(smg_prolongator* P, double* block_vecs);
/* Prolongator::prolong / restrict_vec (src/prolongator.h:77-108) on host
 * arrays: fine 2V complex, coarse (L/bx)(L/by) k complex [block][k]. */
SMG_API smg_status smg_prolongator_prolong(smg_prolongator* P, const double* coarse, double* fine);
SMG_API smg_status smg_prolongator_restrict(smg_prolongator* P, const double* fine, double* coarse);
/* SparseCoarseOp::build(P, A = D^dag D) (src/coarse_op.h:241-279): the
 * 9-point Galerkin operator P^dag D^dag D P, formed directly from D P. */
SMG_API smg_status smg_coarse_op_create(const smg_prolongator* P, smg_dirac* d, smg_coarse_op** out);
SMG_API smg_status smg_coarse_op_destroy(smg_coarse_op* A);
SMG_API smg_status smg_coarse_op_dims(smg_coarse_op* A, int* nbx, int* nby, int* k);
/* SparseCoarseOp::link, [block][dir][ki * k + kj] (src/coarse_op.h:159-166). */
SMG_API smg_status smg_coarse_op_get_links(smg_coarse_op* A, double* links);
/* SparseCoarseOp::apply_to (src/coarse_op.h:282-297) on host arrays. */
SMG_API smg_status smg_coarse_op_apply(smg_coarse_op* A, const double* in, double* out);
/* SparseCoarseOp::solve (src/coarse_op.h:492-547): CG to ||r|| / ||b|| < tol
 * or max_iter iterations, from the deflated guess when deflation pairs are
 * held (smg_coarse_op_setup_deflation). */
SMG_API smg_status smg_coarse_op_solve(smg_coarse_op* A, const double* b, double* x, int max_iter, double tol);
/* SparseCoarseOp::setup_deflation (src/coarse_op.cpp:10-54): TRLM eigenpairs
 * of the operator (see smg_mg_setup_deflation). */
SMG_API smg_status smg_coarse_op_setup_deflation(smg_coarse_op* A, int n_ev, int n_kr, int max_restarts, double tol,
                                                 smg_deflation_info* info);

/* Benchmark support, no reference counterpart: device milliseconds of one
 * application of the level-`level` coarse operator to nrhs right-hand sides
 * in the hierarchy's precision, averaged over `reps` back-to-back
 * applications timed with CUDA events on the context's stream, and the
 * algorithmic HBM bytes of one application (links once, input and output
 * vectors once). */
/* The batched coarse operator of level `level` >= 1 of an F32 hierarchy on
 * host arrays in the device layout, [site][dof][rhs] complex64 with sites
 * lexicographic on the coarse lattice (SparseCoarseOp::apply on nrhs vectors,
 * src/coarse_op.h:282-297).  engine 0: FP32 on the CUDA cores; engine 1: the
 * tensor-core kernel (SMG_UNSUPPORTED unless the level has 16 dofs, a width
 * divisible by 8 and nrhs is a multiple of 32).  dots (optional, per rhs):
 * with w, <out, w> (re, im) and ||out||^2; without w, ||out||^2. */
SMG_API smg_status smg_mg_coarse_apply_batch(smg_mg* mg, int level, int nrhs, int engine, const float* in,
                                             const float* w, float* out, double* dots);
SMG_API smg_status smg_mg_time_coarse_apply(smg_mg* mg, int level, int nrhs, int reps, double* ms, double* bytes);
/* Timing of the fine smoother's kernels (mr_smooth_op, src/smoother.cpp:26-40)
 * on the hierarchy's FP16 work vectors (F32 hierarchy with smoother_half):
 * ms[0] t = D r with ||t||^2 fused, ms[1] A r = D^dag t with ||A r||^2 fused
 * and the MR scalars finished, ms[2] the residual update r' = r - omega A r,
 * ms[3] the pass that adds omega_k r_k of one smoothing into x; each the
 * average of `reps` launches timed with CUDA events on the context's stream
 * after one warm-up pass.  r is formed from b (F32, nrhs a power of two
 * >= 8).  bytes[k] (optional): each kernel's compulsory HBM bytes. */
SMG_API smg_status smg_mg_time_smoother(smg_mg* mg, const smg_field* b, int reps, double* ms, double* bytes);
/* Timing of the coarsest-level solve of the last cycle (SparseCoarseOp::solve,
 * src/coarse_op.h:492-547) on the hierarchy's coarsest work vectors for the
 * cycle's right-hand-side count: ms = the average of `reps` solves timed with
 * CUDA events on the context's stream after one warm-up solve; iters (optional)
 * = the CG iterations of the last solve when it ran as one cooperative launch,
 * else -1.  The hierarchy must have run a cycle (SMG_BAD_ARG otherwise). */
SMG_API smg_status smg_mg_time_coarse_solve(smg_mg* mg, int reps, double* ms, int* iters);

/* fcg_solve / fcg_solve_mg: truncated GCR on A = D^dag D from x = 0
 * (reference src/solvers.cpp:223-300, 803-811), preconditioned by one MG
 * cycle per iteration (mg != NULL) or unpreconditioned (mg == NULL).  The
 * orthogonalisation coefficient is <A p_i, A z> / <A p_i, A p_i>; the
 * reference's conjugate of it (solvers.cpp:261) is used when
 * reference_coefficient != 0.  Runs in the precision of the fields; with an
 * F32 hierarchy and F64 fields the preconditioner runs in FP32 on the
 * normalised residual. */
SMG_API smg_status smg_gcr_solve(smg_dirac* d, smg_mg* mg, const smg_field* rhs, smg_field* x, int max_iter,
                                 double tol, int trunc, int reference_coefficient, smg_solve_result* res);

/* fgmres_solve_generic / fgmres_solve_mg (src/solvers.cpp:555-800): restarted
 * flexible GMRES(restart) on D^dag D with one MG cycle per step (mg != NULL)
 * or none, Ritz harvesting of n_ritz_harvest pairs per cycle (reference
 * default 4) and deflation of later preconditioned vectors with them.
 * Every right-hand side runs its own Arnoldi process; each stops on
 * |g_k+1| / ||b|| < tol inside a cycle or on the true residual at a restart.
 * res->final_residual and res->true_residual are the true ||b - A x|| / ||b||
 * (worst over right-hand sides).  Optional outputs: ritz_values
 * [rhs][3 * n_ritz_harvest] (the Ritz values kept at the end, in list order)
 * and n_ritz[rhs] (how many).  1 <= restart <= 32, n_ritz_harvest <= 8. */
SMG_API smg_status smg_fgmres_solve(smg_dirac* d, smg_mg* mg, const smg_field* rhs, smg_field* x, int restart,
                                    int max_iter, double tol, int n_ritz_harvest, smg_solve_result* res,
                                    double* ritz_values, int* n_ritz);

/* ------------------------------------------------------ multi-lattice batch */

/* Many independent lattices of uneven size on one GPU (no reference
 * counterpart: the reference runs one lattice per process).  Every lattice
 * gets its own context and stream; n_workers host threads take lattices from
 * one queue, largest first, so up to n_workers lattices run at once. */
SMG_API smg_status smg_batch_create(int device, int n_workers, smg_batch** out);
SMG_API smg_status smg_batch_destroy(smg_batch* b);
/* Adds a lattice (links U in the reference layout, 2*L*L complex) with nrhs
 * right-hand sides; id receives its index. */
SMG_API smg_status smg_batch_add(smg_batch* b, int L, const double* U, double mass, double wilson_r, double c_sw,
                                 double mu_t, int nrhs, int* id);
/* Builds every lattice's MG hierarchy with the same parameters, concurrently. */
SMG_API smg_status smg_batch_setup(smg_batch* b, const smg_mg_params* p);
/* Host arrays of a lattice: rhs (nrhs * 2 L^2 complex, uploaded now), and the
 * destinations of x and of the force (2 L^2 doubles) for host_io solves;
 * any may be NULL. */
SMG_API smg_status smg_batch_bind_host(smg_batch* b, int id, const double* rhs, double* x, double* force);
/* Solves D^dag D x = b for every lattice with smg_gcr_solve and its hierarchy
 * (FP32 hierarchy: FP32 GCR inside FP64 defect correction to a true FP64
 * residual below tol) and, with with_force, accumulates F = sum_j F(X_j), the
 * pseudofermion force of S = sum_j phi_j^dag (D^dag D)^-1 phi_j with phi = b.
 * host_io != 0 copies the bound host right-hand sides in and x / force out
 * inside the call.  seconds: wall time of the whole batch.  Returns the worst
 * status over lattices (smg_batch_result gives each). */
SMG_API smg_status smg_batch_solve(smg_batch* b, int max_iter, double tol, int trunc, int with_force, int host_io,
                                   double* seconds);
SMG_API smg_status smg_batch_result(smg_batch* b, int id, smg_solve_result* res, smg_status* status,
                                    double* seconds);
SMG_API smg_status smg_batch_download(smg_batch* b, int id, double* x, double* force);
/* Kernels launched so far by all lattices of the batch. */
SMG_API smg_status smg_batch_kernel_launches(smg_batch* b, uint64_t* n);

/* ------------------------------------------------------------------ forces */

/* fermion_force (reference src/hmc_forces.cpp:134-194 and 198-495): with
 * chi = D X recomputed on the device and never stored, force[mu][s] =
 * -dS/dtheta_mu(s) for S = phi^dag (D^dag D)^-1 phi, X = (D^dag D)^-1 phi.
 * X is a single-RHS F64 field; force is 2*V doubles on the host. */
SMG_API smg_status smg_fermion_force(smg_dirac* d, const smg_field* X, double* force);
/* Forward pass of the pseudofermion action (fermion_action /
 * fermion_action_precond, src/hmc_forces.cpp:113-131): X = (D^dag D)^-1 phi
 * by PCG (mg: preconditioner or NULL) and action[rhs] = Re <phi, X>.  X is
 * what smg_fermion_force (the backward pass) takes. */
SMG_API smg_status smg_fermion_action(smg_dirac* d, smg_mg* mg, const smg_field* phi, smg_field* X, int max_iter,
                                      double tol, double* action, smg_solve_result* res);

/* --------------------------------------------------------------------- HMC */

/* The reference's std::mt19937 passed through an HMC run (momenta, the
 * pseudofermion's eta and the Metropolis draw come from it in the reference's
 * order). */
typedef struct smg_rng smg_rng;
SMG_API smg_status smg_rng_create(uint32_t seed, smg_rng** out);
SMG_API smg_status smg_rng_destroy(smg_rng* rng);
/* std::uniform_real_distribution<double>(0, 1) draw, as the accept step. */
SMG_API smg_status smg_rng_uniform(smg_rng* rng, double* out);
/* n draws of one std::normal_distribution<double>(0, 1) object, as
 * MomentumField::randomise and random_vec make them. */
SMG_API smg_status smg_rng_normal(smg_rng* rng, int64_t n, double* out);

/* HMCParams (reference src/hmc.h:107-119) plus the nested multi-timescale
 * integrator of hmc_trajectory_mg_multiscale (src/hmc_multiscale.cpp:660-710)
 * with the gauge force as its cheap inner force:
 *   n_inner = 0: hmc_trajectory's integrator (src/hmc_trajectory.cpp:243-409),
 *                leapfrog or Omelyan (lambda = 0.1932) over gauge + fermion
 *                forces with n_steps steps of tau / n_steps;
 *   n_inner > 0: the fermion force drives the outer integrator (n_steps
 *                steps, leapfrog or Omelyan) and every outer momentum kick is
 *                separated by an inner leapfrog of n_inner steps on the gauge
 *                force alone.
 * mixed_precision selects smg_cg_solve_mixed for every solve (otherwise FP64
 * CG). */
typedef struct {
    double beta;
    double tau;
    int n_steps;
    int omelyan;
    int n_inner;
    int cg_maxiter;
    double cg_tol;
    double c_sw;
    double mu_t;
    int force_accept;
    int mixed_precision;
    int use_eo;  /* the reference's even-odd path: Schur-complement pseudofermion
                    phi_o = M^dag eta_o, CG on M^dag M, eo_fermion_force and
                    H += -2 log det D_ee (src/hmc_trajectory.cpp:59-165); with
                    n_inner == 0 it integrates with leapfrog as the reference does */
} smg_hmc_params;

/* HMCResult (reference src/hmc.h:121-129) plus the plaquette after the
 * trajectory (accepted or restored) and the number of solves. */
typedef struct {
    int accepted;
    double dH, dKE, dSG, dSF;
    int total_cg_iters;
    int solves;
    double plaquette;
    double dLD;  /* change of -2 log det D_ee (even-odd path; 0 otherwise) */
} smg_hmc_result;

SMG_API smg_status smg_hmc_params_default(smg_hmc_params* p);
/* hmc_trajectory (reference src/hmc_trajectory.cpp:38-235, full-lattice
 * path): momenta pi ~ N(0,1) from rng, phi = D^dag eta with eta = random_vec,
 * H = KE + S_G + S_F with S_F = Re <phi, (D^dag D)^-1 phi>, molecular
 * dynamics with the device forces, Metropolis with rng; a rejected
 * trajectory restores the links.  The gauge handle is updated in place;
 * gauge, momenta, forces and fields stay on the device. */
SMG_API smg_status smg_hmc_trajectory(smg_gauge* g, double mass, double wilson_r, const smg_hmc_params* p,
                                      smg_rng* rng, smg_hmc_result* res);

/* ReversibilityResult (reference src/hmc.h:402-408) plus the number of solves. */
typedef struct {
    double gauge_delta;  /* ||U_end - U_start|| / ||U_start|| */
    double mom_delta;    /* ||-pi_end - pi_start|| / ||pi_start|| */
    double dH_forward;
    double dH_backward;  /* -dH_forward for a reversible integrator */
    int total_cg_iters;
    int solves;
} smg_reversibility_result;

/* reversibility_test_plain (reference src/hmc_trajectory.cpp:416-509): the
 * pseudofermion phi = D^dag eta and then the momenta are drawn from rng, the
 * molecular dynamics of smg_hmc_trajectory runs forward, the momenta are
 * negated, it runs again, and the links and momenta are compared with the
 * start.  The links at entry are restored before return.  The integrator is
 * the one smg_hmc_trajectory uses for *p (n_inner and use_eo included; the
 * reference's test covers n_inner = 0, use_eo = 0). */
SMG_API smg_status smg_hmc_reversibility(smg_gauge* g, double mass, double wilson_r, const smg_hmc_params* p,
                                         smg_rng* rng, smg_reversibility_result* res);

/* Outer integrators of hmc_trajectory_mg_multiscale (OuterIntegrator,
 * reference src/hmc.h:327-336). */
typedef enum {
    SMG_OUTER_LEAPFROG = 0,
    SMG_OUTER_OMELYAN = 1,  /* 2MN, lambda = 0.1932 */
    SMG_OUTER_FGI = 2,      /* force-gradient PQPQP, lambda = 1/6, xi = 1/72 */
    SMG_OUTER_FGI_QPQPQ = 3 /* force-gradient QPQPQ */
} smg_outer_integrator;

/* MGMultiScaleParams (reference src/hmc.h:338-357) without the research
 * options (deflation refresh, perturbative MG refresh, eigenspace tracking,
 * even-odd), which stay at their defaults (off). */
typedef struct {
    double beta;
    double tau;
    int n_outer;
    int n_inner;
    int cg_maxiter;
    double cg_tol;
    int inner_smooth;  /* MR steps before and after the low-mode projection (0 = raw projection) */
    int outer_type;    /* smg_outer_integrator */
    double c_sw;
    double mu_t;
} smg_ms_params;

/* MGMultiScaleResult (reference src/hmc.h:359-367) without the wall-clock
 * split, plus the plaquette after the trajectory and the number of solves. */
typedef struct {
    int accepted;
    double dH, dKE, dSG, dSF;
    int highmode_cg_iters; /* every MG-preconditioned CG iteration of the trajectory */
    int lowmode_force_evals;
    int solves;
    double plaquette;
} smg_ms_result;

/* coarse_lowmode_force (reference src/hmc_multiscale.cpp:237-276): with
 * smooth_iters > 0, x = MR(D^dag D, phi, from 0), x += lowmode_solution of
 * phi - D^dag D x, x = MR(D^dag D, phi, from x); with smooth_iters = 0 the
 * low-mode solution of phi itself; force = fermion_force(D, x) as host
 * [mu][s] doubles.  The low-mode solution uses mg's level-0 prolongator and
 * deflation space. */
SMG_API smg_status smg_coarse_lowmode_force(smg_dirac* d, smg_mg* mg, const smg_field* phi, int smooth_iters,
                                            double* force);

/* n_outer = 4, n_inner = 5, cg_maxiter = 500, cg_tol = 1e-10,
 * inner_smooth = 3, leapfrog, c_sw = mu_t = 0, beta = 4, tau = 1. */
SMG_API smg_status smg_ms_params_default(smg_ms_params* p);

/* hmc_trajectory_mg_multiscale (reference src/hmc_multiscale.cpp:340-886,
 * without tracking, forecasting or refreshes): the outer integrator kicks with
 * the gauge force plus the fermion force (MG-preconditioned CG with the
 * hierarchy mg) minus the low-mode force, the inner leapfrog (n_inner steps)
 * with the low-mode force alone; the low-mode force is the fermion force of
 * coarse_lowmode_force (src/hmc_multiscale.cpp:237-276) built from mg's
 * level-0 prolongator and deflation space.  mg must have been built on a
 * Dirac operator over the gauge handle g; its coarse operators are not
 * rebuilt during the trajectory (smg_mg_rebuild and smg_mg_deflation_rr
 * between trajectories do what the reference's MG-HMC driver does).  As in the
 * reference the momenta are drawn first and the pseudofermion is drawn twice,
 * the second draw used. */
SMG_API smg_status smg_hmc_mg_multiscale(smg_gauge* g, double mass, double wilson_r, const smg_ms_params* p,
                                         smg_mg* mg, smg_rng* rng, smg_ms_result* res);
/* reversibility_test_mg_multiscale (reference src/hmc_multiscale.cpp:963-
 * 1000): momenta then one pseudofermion from rng, forward molecular dynamics,
 * momentum flip, backward; the links at entry are restored.  As in the
 * reference the forces use mu_t = 0 and FGI_QPQPQ runs as FGI. */
SMG_API smg_status smg_hmc_mg_multiscale_reversibility(smg_gauge* g, double mass, double wilson_r,
                                                       const smg_ms_params* p, smg_mg* mg, smg_rng* rng,
                                                       smg_reversibility_result* res);

/* --------------------------------------------------- force verification */

#define SMG_VERIFY_LINKS 20

/* Outcome of smg_verify_forces: per tested link (mu, site) the analytic and
 * finite-difference gauge and fermion forces, and the maxima the reference
 * prints (max |ana - num| and that over max |ana|). */
typedef struct {
    int passed, gauge_passed, fermion_passed;
    double gauge_max_err, gauge_rel, fermion_max_err, fermion_rel;
    int n_links;
    int mu[SMG_VERIFY_LINKS], site[SMG_VERIFY_LINKS];
    double gf_ana[SMG_VERIFY_LINKS], gf_num[SMG_VERIFY_LINKS];
    double ff_ana[SMG_VERIFY_LINKS], ff_num[SMG_VERIFY_LINKS];
} smg_force_check;

/* verify_forces (reference src/hmc_forces.cpp:869-981): the device's gauge
 * force and pseudofermion force (full D^dag D or, with use_eo, the Schur
 * complement with -2 log det D_ee) against central differences (eps = 1e-5)
 * of the actions at the reference's 20 links (mu = t % 2,
 * s = (7 t + 13 (t / 2)) % V), with its pseudofermion (random_vec from
 * std::mt19937(12345)); passes when both relative errors are below
 * err_threshold (the reference's callers use 1e-4). */
SMG_API smg_status smg_verify_forces(smg_gauge* g, double beta, double mass, double wilson_r, int max_iter,
                                     double tol, double c_sw, int use_eo, double err_threshold, double mu_t,
                                     smg_force_check* out);

/* ------------------------------------------------------------ gauge files */

/* GaugeHeader (reference src/hmc.h:19-25): the 32-byte header of the "SWNG"
 * gauge file, little-endian, followed by U[0][0..V) and U[1][0..V) as
 * complex128 (save_gauge / load_gauge, src/hmc_forces.cpp:18-62). */
typedef struct {
    uint32_t magic; /* 0x53574E47 */
    uint32_t L;
    double beta;
    double mass;
    double avg_plaq;
} smg_gauge_header;

/* save_gauge: writes hdr {magic, L, beta, mass, avg_plaq} and the links. */
SMG_API smg_status smg_host_gauge_write_swng(const char* path, int L, const double* U, double beta, double mass,
                                             double avg_plaq);
/* load_gauge: reads the header (SMG_BAD_ARG on a wrong magic, or on an L other
 * than L_expected when L_expected > 0) and, when U != NULL, the links divided
 * by their modulus as the reference does after reading.  Reading the links
 * needs L_expected > 0 (U must hold 4 * L_expected^2 doubles); to learn L from
 * a file, call first with U == NULL and read hdr->L. */
SMG_API smg_status smg_host_gauge_read_swng(const char* path, int L_expected, smg_gauge_header* hdr, double* U);
/* GaugeField::save / load (src/gauge.h:38-57): int32 V, then the links. */
SMG_API smg_status smg_host_gauge_write_raw(const char* path, int L, const double* U);
SMG_API smg_status smg_host_gauge_read_raw(const char* path, int L, double* U);
/* The same formats from and into a device gauge handle; smg_gauge_save writes
 * the handle's plaquette into the header. */
SMG_API smg_status smg_gauge_save(smg_gauge* g, double beta, double mass, const char* path);
SMG_API smg_status smg_gauge_load(smg_gauge* g, const char* path, smg_gauge_header* hdr);

/* -------------------------------------------------------- host utilities */

/* Seeded synthetic inputs drawn with the C++ standard library generators the
 * reference uses (std::mt19937 + std::normal_distribution<double>), so the
 * same seed gives the reference's own numbers.
 * Gauge: theta_mu(s) ~ N(0, 1/beta) i.i.d. drawn mu-major then site order,
 * U = exp(i theta).  Vector: the order of random_vec as GCC on x86-64
 * compiles it (reference src/linalg.cpp:44-48), which draws each entry's
 * imaginary part before its real part. */
SMG_API smg_status smg_host_gauge_normal(int L, double beta, uint32_t seed, double* U);
SMG_API smg_status smg_host_random_vec(int64_t n_complex, uint32_t seed, double* v);

#ifdef __cplusplus
}
#endif
#endif /* SMG_GPU_H */
