/*
 * starpu_cublas_v2.h -- kept so that sources written for StarPU include it unchanged; the
 * declarations it would add live in starpu_cuda.h (included by starpu.h).
 * The GB300 runtime does not link the vendor libraries.
 */
#ifndef STARPU_CUBLAS_V2_H
#define STARPU_CUBLAS_V2_H
#include "starpu.h"
#endif
