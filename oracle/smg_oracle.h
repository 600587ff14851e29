/* ORACLE TEST INFRASTRUCTURE — not part of the product.
 *
 * CPU restatement in plain C (OpenMP) of the reference's Wilson-clover Dirac
 * operator and multigrid solve path (cpviolator/Schwinger_MG).  Only the test
 * suite, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, as
 * the checker; the product never links it.
 *
 * Parity pin: tests/test_oracle_pin.py checks every function here against the
 * reference's own code (oracle/_ref/libsmg_ref.so, compiled from the
 * reference sources by oracle/Makefile) and against tests/golden/ fixtures
 * that script generated from the reference.
 *
 * Arrays use the reference layouts: complex numbers interleaved (re, im);
 * spinor v[2*s + spin] with s = x + L*y; links U[mu][s]; force F[mu][s];
 * block vectors [block][k][2*bs*bs]; coarse links [block][dir][ki*k + kj]. */
#ifndef SMG_ORACLE_H
#define SMG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

void orc_set_threads(int n);
int orc_get_threads(void);

void orc_clover(int L, const double* U, double* F01);
double orc_avg_plaq(int L, const double* U);
/* op: 0 D, 1 D^dag, 2 D^dag D, 3 g5 D */
void orc_dirac(int L, const double* U, double m, double r, double csw, double mu, int op, const double* src,
               double* dst);
int orc_cg(int L, const double* U, double m, double r, double csw, double mu, const double* b, double* x,
           int max_iter, double tol, double* final_res);
void orc_gauge_force(int L, const double* U, double beta, double* F);
double orc_gauge_action(int L, const double* U, double beta);
void orc_fermion_force(int L, const double* U, double m, double r, double csw, double mu, const double* X,
                       double* F);
void orc_mr_smooth(int L, const double* U, double m, double r, double csw, double mu, const double* b, double* x,
                   int niter);
void orc_near_null_space(int L, const double* U, double m, double r, double csw, double mu, int k, int iters,
                         const double* init, double* out);
void orc_prolongator_build(int L, int bs, int k, const double* null_vecs, double* block_vecs);
void orc_prolong(int L, int bs, int k, const double* block_vecs, const double* coarse, double* fine);
void orc_restrict(int L, int bs, int k, const double* block_vecs, const double* fine, double* coarse);
void orc_sparse_coarse_build(int L, const double* U, double m, double r, double csw, double mu, int bs, int k,
                             const double* block_vecs, double* links);
void orc_sparse_coarse_apply(int nbx, int nby, int k, const double* links, const double* src, double* dst);
int orc_sparse_coarse_cg(int nbx, int nby, int k, const double* links, const double* b, double* x, int max_iter,
                         double tol);

/* Two-level MG on A = D^dag D with a given level-0 prolongator (block_vecs)
 * and 9-point coarse operator (links): V-cycle of mg_cycle
 * (reference src/multigrid.cpp:43-102) with MR smoothing and a coarse CG
 * solve (reference src/coarse_op.h:492-547 without deflation). */
typedef struct {
    int L, bs, k;
    double m, r, csw, mu;
    int pre_smooth, post_smooth;
    int coarse_max_iter;
    double coarse_tol;
} orc_mg2_params;

void orc_mg2_precondition(const orc_mg2_params* p, const double* U, const double* block_vecs, const double* links,
                          const double* b, double* out);
/* fcg_solve (truncated GCR, reference src/solvers.cpp:223-300) with the
 * two-level preconditioner; returns iterations.  ref_coeff selects the
 * reference's orthogonalisation coefficient (see smg_oracle.c). */
int orc_mg2_gcr(const orc_mg2_params* p, const double* U, const double* block_vecs, const double* links,
                const double* b, double* x, int max_iter, double tol, int trunc, int ref_coeff,
                double* final_res);

/* N-level MG on a given hierarchy (block vectors and coarse operators as
 * returned by smg_mg_get_prolongator / smg_mg_get_coarse_op).  links[0] is
 * unused (level 0 is D^dag D). */
#define ORC_MAX_LEVELS 6
typedef struct {
    int n_levels, L;
    double m, r, csw, mu;
    int block[ORC_MAX_LEVELS - 1][2];
    int nc[ORC_MAX_LEVELS - 1];
    const double* block_vecs[ORC_MAX_LEVELS - 1];
    const double* links[ORC_MAX_LEVELS];
    int pre_smooth, post_smooth, w_cycle, coarse_max_iter;
    double coarse_tol;
} orc_mgN_params;

void orc_mgN_precondition(const orc_mgN_params* p, const double* U, const double* b, double* out);
int orc_mgN_gcr(const orc_mgN_params* p, const double* U, const double* b, double* x, int max_iter, double tol,
                int trunc, double* final_res, double* seconds);

/* Hierarchy set-up on the CPU (the reference's build_mg_hierarchy with a
 * geometric aggregate at every level and direct Galerkin products; see
 * smg_oracle.c).  block_vecs[l] receives level l's block vectors
 * [agg][i][loc * ndof_l + j], links[l + 1] level l + 1's operator in the
 * SparseCoarseOp layout [site][dir][i * nc + j], null0 (optional) the level-0
 * null vectors; the caller sizes every array.  Returns 0, or < 0 for a bad
 * geometry. */
typedef struct {
    int n_levels, L;
    double m, r, csw, mu;
    int block[ORC_MAX_LEVELS - 1][2];
    int nvec[ORC_MAX_LEVELS - 1];
    int chiral_split, null_iters, null_mr_steps;
    uint32_t seed;
} orc_mgN_setup_params;

int orc_mgN_setup(const orc_mgN_setup_params* p, const double* U, double* const* block_vecs, double* const* links,
                  double* null0);

/* Seeded inputs (oracle/inputs.cpp): random_vec(n, std::mt19937(seed)) and
 * links U = exp(i theta), theta ~ N(0, 1/beta). */
void orc_random_vec(long n, uint32_t seed, double* v);
void orc_gauge_normal(int L, double beta, uint32_t seed, double* U);

/* CPU timing of the restatement (bench.py's CPU baseline): seconds for `reps`
 * applications of D (op 0) or D^dag D (op 2) to nrhs spinors, and for one CG
 * solve; the operator is set up outside the timed region. */
double orc_time_dirac(int L, const double* U, double m, double r, double csw, double mu, int op, int nrhs,
                      const double* src, double* dst, int reps);
double orc_time_cg(int L, const double* U, double m, double r, double csw, double mu, const double* b, double* x,
                   int max_iter, double tol, int* iters);

#ifdef __cplusplus
}
#endif
#endif
