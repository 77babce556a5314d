/*
 * starpu_cusolver.h -- kept so that sources written for StarPU include it unchanged; the
 * declarations it would add live in starpu_cuda.h (included by starpu.h).
 * The GB300 runtime does not link the vendor libraries.
 */
#ifndef STARPU_CUSOLVER_H
#define STARPU_CUSOLVER_H
#include "starpu.h"
#endif
