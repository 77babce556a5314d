/*
 * starpu_sched_ctx.h -- kept so that sources written for StarPU include it unchanged; its
 * declarations are part of starpu.h in this implementation.
 */
#ifndef STARPU_SCHED_CTX_H
#define STARPU_SCHED_CTX_H
#include "starpu.h"
#endif
