/* ORACLE TEST INFRASTRUCTURE — not part of the product.
 *
 * Stand-ins for the two FEAST Fortran entry points the reference declares
 * (reference src/feast_solver.cpp:12-18).  FEAST (certik/feast, branch
 * master, fetched by the reference's CMake at configure time and not vendored)
 * is absent here; it only serves the optional `--eigensolver feast` null-space
 * path, which is off the solve path (default eigensolver "trlm",
 * reference src/config.h:36).  zfeast_hrci_ reports failure (info = -1) so a
 * FEAST call in the reference returns no eigenpairs instead of computing. */
void feastinit_(int* fpm) {
    for (int i = 0; i < 64; ++i) fpm[i] = 0;
}

void zfeast_hrci_(int* ijob, int* N, double* Ze, double* work, double* workc, double* zAq, double* zSq, int* fpm,
                  double* epsout, int* loop, double* Emin, double* Emax, int* M0, double* lambda, double* q,
                  int* mode, double* res, int* info) {
    (void)N; (void)Ze; (void)work; (void)workc; (void)zAq; (void)zSq; (void)fpm; (void)epsout;
    (void)Emin; (void)Emax; (void)M0; (void)lambda; (void)q; (void)res;
    *ijob = 0;
    *loop = 0;
    *mode = 0;
    *info = -1;
}
