/*
 * starpu_thread_util.h -- kept so that sources written for StarPU include it unchanged; its
 * declarations are part of starpu.h in this implementation.
 */
#ifndef STARPU_THREAD_UTIL_H
#define STARPU_THREAD_UTIL_H
#include "starpu.h"
#endif
