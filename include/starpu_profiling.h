/*
 * starpu_profiling.h -- kept so that sources written for StarPU include it unchanged; its
 * declarations are part of starpu.h in this implementation.
 */
#ifndef STARPU_PROFILING_H
#define STARPU_PROFILING_H
#include "starpu.h"
#endif
