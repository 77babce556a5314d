/*
 * starpu_fxt.h -- kept so that sources written for StarPU include it unchanged; its
 * declarations are part of starpu.h in this implementation.
 */
#ifndef STARPU_FXT_H
#define STARPU_FXT_H
#include "starpu.h"
#endif
