/*
 * starpu_config.h -- build configuration of the GB300 StarPU-API runtime.
 *
 * The runtime behind these headers is libstarpu_gb300.so: one host (CPU
 * workers) and CUDA devices of the GB300 (sm_103a).  Code compiled with
 * -DSTARPU_GB300_CPU_ONLY sees a CPU-only configuration (no STARPU_USE_CUDA),
 * which is how CPU-only codelet files are built against the same headers.
 */
#ifndef STARPU_CONFIG_H
#define STARPU_CONFIG_H

#define STARPU_MAJOR_VERSION 1
#define STARPU_MINOR_VERSION 4
#define STARPU_RELEASE_VERSION 99

#ifndef STARPU_GB300_CPU_ONLY
#define STARPU_USE_CUDA 1
#endif
#define STARPU_USE_CPU 1
#define STARPU_GB300 1

/* CPU codelets of the examples call a Fortran BLAS (sgemm_, ...): OpenBLAS */
#define STARPU_OPENBLAS 1

#define STARPU_MAXNODES 4
#define STARPU_NMAXBUFS 8
#define STARPU_MAXIMPLEMENTATIONS 4
#define STARPU_NMAXWORKERS 256
#define STARPU_MAXCPUS 256
#define STARPU_MAXCUDADEVS 8
#define STARPU_NMAX_SCHED_CTXS 10

#endif /* STARPU_CONFIG_H */
