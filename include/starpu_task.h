/*
 * starpu_task.h -- kept so that sources written for StarPU include it unchanged; its
 * declarations are part of starpu.h in this implementation.
 */
#ifndef STARPU_TASK_H
#define STARPU_TASK_H
#include "starpu.h"
#endif
