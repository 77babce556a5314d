/*
 * starpu_bound.h -- kept so that sources written for StarPU include it unchanged; its
 * declarations are part of starpu.h in this implementation.
 */
#ifndef STARPU_BOUND_H
#define STARPU_BOUND_H
#include "starpu.h"
#endif
