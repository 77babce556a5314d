/*
 * starpu_gb300_solver.h -- SPD solve entry points of the GB300 kernel layer.
 *
 * The reference has no solve, no mixed precision, no batching and no serving
 * (its Cholesky is FP32 factorisation only: examples/cholesky/cholesky_kernels.c:53-55);
 * these entry points extend the factorisation of starpu_gb300_kernels.h to
 * A X = B for SPD A with LAPACK dposv / dsposv semantics.  Same conventions
 * as starpu_gb300_kernels.h: column-major, void* stream, no synchronisation,
 * no device allocation (work buffers are passed in).
 */
#ifndef STARPU_GB300_SOLVER_H
#define STARPU_GB300_SOLVER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- synthetic inputs (benchmarks and tests) ----------------
 * Row i of B ~ N(0,1) from PCG64 stream i+1 of `seed` (Box-Muller pairs);
 * right-hand-side column j ~ U[-1,1] from PCG64 stream 2^40+j.
 * gen_spd_gram: A = B B^T / n + alpha I (full symmetric), `work` n*n doubles. */
int starpu_gb300_gen_normal(void *stream, int rows, int cols, uint64_t seed, double *B, int ldb);
int starpu_gb300_gen_uniform_rhs(void *stream, int n, int nrhs, uint64_t seed, double *B, int ldb);
int starpu_gb300_gen_spd_gram(void *stream, int n, uint64_t seed, double alpha, double *A, int lda, double *work);

#ifdef __cplusplus
}
#endif

#endif /* STARPU_GB300_SOLVER_H */
