/*
 * starpu_data_interfaces.h -- kept so that sources written for StarPU include it unchanged; its
 * declarations are part of starpu.h in this implementation.
 */
#ifndef STARPU_DATA_INTERFACES_H
#define STARPU_DATA_INTERFACES_H
#include "starpu.h"
#endif
