/*
 * sa_matched_filter.h -- C ABI of libsa_matched_filter.so: the four entry
 * points of the reference's libmatched_filter.so (declared at
 * sa_library/matched_filter.c:53-56 and bound by
 * sa_library/matched_filter_c.py:17-34) under the reference's own names, so
 * that the library can be linked or symlinked in its place.  Each forwards
 * to the GPU matched filter of libsa_cuda.so (include/sa_finder.h): the
 * handle is an saFilterCreate handle, the arrays are host arrays as in the
 * reference, and failures print and are kept for saGetLastError.
 */
#ifndef SA_MATCHED_FILTER_H
#define SA_MATCHED_FILTER_H

#ifdef __cplusplus
extern "C" {
#endif

/* matched_filter.c:66 cleanup */
void cleanup(void *flt);
/* matched_filter.c:93 convolve */
void convolve(void *flt, double *image, double *result);
/* matched_filter.c:118 convolveMemo */
void convolveMemo(void *flt, double *image, double *result);
/* matched_filter.c:163 initialize (psf recentred, x_size x y_size) */
void *initialize(double *psf, double max_diff, int x_size, int y_size, int estimate);

#ifdef __cplusplus
}
#endif

#endif
