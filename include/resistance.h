/* The diagonal resistance matrix of the reference's include/resistance.h
 * (struct layout only, resistance.h:92-98): n values, R[i][i] =
 * diagonal[i].  The reference's resistance functions stay the reference's;
 * the drop-in uses the struct in its Matrix Market export. */
#ifndef PEEC_RESISTANCE_H
#define PEEC_RESISTANCE_H

#include <stddef.h>

typedef struct {
    size_t n;
    double *diagonal;
} ResistanceMatrix;

#endif
