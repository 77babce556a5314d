/*
 * starpu_cuda.h -- CUDA worker API (StarPU include/starpu_cuda.h subset) and
 * the vendor-library handle hooks the drivers call.
 *
 * A CUDA codelet enqueues its work on starpu_cuda_get_local_stream() (the
 * stream of the calling CUDA worker, or of the capture in progress when the
 * runtime records a whole task graph) and, with STARPU_CUDA_ASYNC in
 * cuda_flags, returns without synchronising.
 *
 * The cuBLAS / cuSOLVER / hipBLAS / hipSOLVER init and shutdown calls exist so
 * that drivers written for the reference link unchanged; this runtime's
 * codelets call the GB300 kernel layer (starpu_gb300_kernels.h) instead of
 * the vendor libraries, so these are no-ops.
 */
#ifndef STARPU_CUDA_H
#define STARPU_CUDA_H

#include "starpu_config.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifdef STARPU_USE_CUDA
#include <cuda_runtime.h>
cudaStream_t starpu_cuda_get_local_stream(void);
void starpu_cuda_report_error(const char *func, const char *file, int line, cudaError_t status);
#define STARPU_CUDA_REPORT_ERROR(status) starpu_cuda_report_error(__func__, __FILE__, __LINE__, status)
#endif

void starpu_cublas_init(void);
void starpu_cublas_shutdown(void);
void starpu_cublas_set_stream(void);
void starpu_cusolver_init(void);
void starpu_cusolver_shutdown(void);
void starpu_hipblas_init(void);
void starpu_hipblas_shutdown(void);
void starpu_hipsolver_init(void);
void starpu_hipsolver_shutdown(void);

#ifdef __cplusplus
}
#endif

#endif /* STARPU_CUDA_H */
