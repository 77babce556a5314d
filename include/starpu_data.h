/*
 * starpu_data.h -- kept so that sources written for StarPU include it unchanged; its
 * declarations are part of starpu.h in this implementation.
 */
#ifndef STARPU_DATA_H
#define STARPU_DATA_H
#include "starpu.h"
#endif
