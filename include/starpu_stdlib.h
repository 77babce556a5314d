/*
 * starpu_stdlib.h -- kept so that sources written for StarPU include it unchanged; its
 * declarations are part of starpu.h in this implementation.
 */
#ifndef STARPU_STDLIB_H
#define STARPU_STDLIB_H
#include "starpu.h"
#endif
