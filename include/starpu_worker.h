/*
 * starpu_worker.h -- kept so that sources written for StarPU include it unchanged; its
 * declarations are part of starpu.h in this implementation.
 */
#ifndef STARPU_WORKER_H
#define STARPU_WORKER_H
#include "starpu.h"
#endif
