/*
 * sa_ia_utilities.h -- C ABI of libsa_ia_utilities.so: every entry point of
 * the reference's libia_utilities.so (declared at
 * sa_library/ia_utilities.c:41-49 and bound by
 * sa_library/ia_utilities_c.py:16-87) under the reference's own names, so
 * that the library can be symlinked in its place.  Each forwards to the GPU
 * implementation in libsa_cuda.so (include/sa_finder.h); arrays are host
 * arrays as in the reference, and the flmData layout is the reference's.
 */
#ifndef SA_IA_UTILITIES_H
#define SA_IA_UTILITIES_H

#include <stdint.h>

#include "sa_finder.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ia_utilities.c:58 */
int calcMaxPeaks(saFlmData *flm_data);
/* ia_utilities.c:82 (the handle is a point set, not a tree) */
void *createKDTree(double *x, double *y, int n);
/* ia_utilities.c:105 */
void findLocalMaxima(saFlmData *flm_data, double *z, double *y, double *x, double *h);
/* ia_utilities.c:166 */
void freeKDTree(void *kd);
/* ia_utilities.c:221 */
int markDimmerPeaks(double *x, double *y, double *h, int32_t *status, double r_removal, double r_neighbors, int np);
/* ia_utilities.c:292 */
int markLowSignificancePeaks(double *x, double *y, double *sig, int32_t *status, double min_sig,
                             double r_neighbors, int np);
/* ia_utilities.c:347 */
void nearestKDTree(void *kd, double *x, double *y, double *dist, int32_t *index, double radius, int n);
/* ia_utilities.c:401 */
void runningIfHasNeighbors(double *c_x, double *c_y, double *n_x, double *n_y, int32_t *status, double radius,
                           int nc, int nn);

#ifdef __cplusplus
}
#endif

#endif
