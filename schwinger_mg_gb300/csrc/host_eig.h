// Small dense eigenproblems solved on the host (the k x k projected matrices of
// the Krylov and Rayleigh-Ritz methods; the reference's lanczos_eigen /
// jacobi_eigen, src/eigensolver_core.cpp:12-270, play the same role).
#pragma once
#include <complex>
#include <vector>

// Eigen-decomposition of a Hermitian n x n matrix A (column-major, A[j * n + i] = A(i, j)).
// Eigenvalues ascending in vals; column c of vecs (vecs[c * n + i]) is the unit eigenvector of vals[c].
void hermitian_eig(int n, std::vector<std::complex<double>> A, std::vector<double>& vals,
                   std::vector<std::complex<double>>& vecs);
