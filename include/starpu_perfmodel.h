/*
 * starpu_perfmodel.h -- kept so that sources written for StarPU include it unchanged; its
 * declarations are part of starpu.h in this implementation.
 */
#ifndef STARPU_PERFMODEL_H
#define STARPU_PERFMODEL_H
#include "starpu.h"
#endif
