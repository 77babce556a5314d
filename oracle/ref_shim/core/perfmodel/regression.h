/*
 * ORACLE build helper (test infrastructure only).  Stands in for the
 * reference's internal header of the same path so that its
 * src/core/perfmodel/regression.c compiles on its own, unchanged, into
 * oracle/_ref/libref_regression.so: the history entry and list types with
 * the fields that file reads (size, mean, nsample; next, entry), the three
 * helper macros it uses, and the prototype it defines.
 */
#ifndef GB300_REF_SHIM_REGRESSION_H
#define GB300_REF_SHIM_REGRESSION_H

#include <assert.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct starpu_perfmodel_history_entry {
    double mean;
    size_t size;
    unsigned nsample;
};

struct starpu_perfmodel_history_list {
    struct starpu_perfmodel_history_list *next;
    struct starpu_perfmodel_history_entry *entry;
};

#define _STARPU_MALLOC(ptr, size) ((ptr) = malloc(size))
#define STARPU_ASSERT(x) assert(x)
#define STARPU_MIN(a, b) ((a) < (b) ? (a) : (b))

int _starpu_regression_non_linear_power(struct starpu_perfmodel_history_list *ptr, double *a, double *b, double *c);

#endif
