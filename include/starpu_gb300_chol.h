/*
 * starpu_gb300_chol.h -- the GB300 Cholesky codelet library
 * (libstarpu_gb300_chol.so), a drop-in for examples/cholesky/cholesky_kernels.c.
 *
 * It defines what the reference's cholesky.h declares extern: the codelets
 * cl_potrf / cl_trsm / cl_syrk / cl_gemm (and the _gpu aliases), the history
 * perfmodels chol_model_potrf / _trsm / _syrk / _gemm, the `scratch` and
 * `devInfo` handles (unused: the GB300 POTRF needs no workspace) and
 * cholesky_kernel_init() / cholesky_kernel_fini().  Link a driver with
 *   -lstarpu_gb300_chol -lstarpu_gb300
 * The reference never reports a failed factorisation (cholesky_kernels.c:351-354
 * writes devInfo but nobody reads it); this library adds the query below
 * without changing any existing signature.
 */
#ifndef STARPU_GB300_CHOL_H
#define STARPU_GB300_CHOL_H

#ifdef __cplusplus
extern "C" {
#endif

/* Waits for the submitted tasks, then returns the LAPACK-style info of the
 * first non-positive pivot met by any POTRF tile since the last reset
 * (0 = every tile factored); reset != 0 clears it. */
int starpu_gb300_chol_status(int reset);

#ifdef __cplusplus
}
#endif

#endif /* STARPU_GB300_CHOL_H */
