// Internal interface between the multigrid hierarchy (mg.cu), its coarse-grid
// deflation space (deflation.cu) and the multi-timescale HMC (hmc.cu).
#pragma once
#include <vector>

#include "smg_internal.h"
#include "vec.cuh"

// Eigenpairs of a coarse operator, by default the level-1 A_c = P^dag (D^dag D) P (SparseCoarseOp::defl_vecs /
// defl_vals, reference src/coarse_op.h:168-200; CoarseDeflState, src/hmc.h:307-324).  Vectors
// are level-1 coarse vectors of one right-hand side ([site][dof], sites lexicographic on the
// coarse lattice, the reference's c[b * k + kv]), stored contiguously one after the other.
struct MgDeflation {
    int level = 1;     // the level whose operator the pairs belong to
    int n = 0;         // number of eigenpairs held
    int cap = 0;       // vectors allocated
    int64_t dim = 0;   // complex entries per vector
    cx<double>* V64 = nullptr;
    cx<float>* V32 = nullptr;    // FP32 copy for the F32 coarsest solve
    double* inv = nullptr;       // device [cap]: 1 / lambda_i, 0 where lambda_i <= 1e-14
    std::vector<double> vals;    // host eigenvalues, ascending
    // scratch of the initial guess: per (vector, rhs) partial sums and coefficients
    double* part = nullptr;
    size_t part_doubles = 0;
    cx<double>* coef = nullptr;  // [cap][32]
    // scratch of the low-mode solution: two level-1 vectors
    cx<double>* c_in = nullptr;
    cx<double>* c_out = nullptr;
};

void smg_defl_free(MgDeflation& d);

// x = sum_i v_i (v_i^dag b) / lambda_i for every right-hand side of the coarse vectors b and x
// (the deflated initial guess of SparseCoarseOp::solve, src/coarse_op.h:492-509)
template <typename T>
smg_status smg_defl_guess(smg_context* ctx, MgDeflation& d, VecView<T> b, VecView<T> x);

// Level-1 helpers provided by mg.cu for single right-hand-side FP64 vectors
struct smg_mg;
MgDeflation& smg_mg_defl(smg_mg* mg);
smg_context* smg_mg_ctx(smg_mg* mg);
smg_dirac* smg_mg_dirac(smg_mg* mg);
int smg_mg_nlevels(const smg_mg* mg);
int64_t smg_mg_level_dim(const smg_mg* mg, int l);  // complex entries of a level-l vector (l >= 1)
smg_status smg_mg_apply_f64(smg_mg* mg, int l, const cx<double>* x, cx<double>* y);          // A_l x
smg_status smg_mg_restrict0_f64(smg_mg* mg, const smg_field* fine, cx<double>* coarse);      // P^dag f
smg_status smg_mg_prolong0_f64(smg_mg* mg, const cx<double>* coarse, smg_field* fine);       // P c
void smg_mg_drop_cycle_graph(smg_mg* mg);  // the captured cycle is re-captured on its next use

// x = P sum_i v_i (v_i^dag P^dag phi) / lambda_i for single-RHS F64 fields (deflation.cu)
smg_status smg_mg_lowmode_internal(smg_mg* mg, const smg_field* phi, smg_field* x);
