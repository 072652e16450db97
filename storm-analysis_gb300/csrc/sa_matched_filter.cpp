// sa_matched_filter.cpp -- libsa_matched_filter.so: the reference-named
// matched-filter entry points (include/sa_matched_filter.h), forwarding to
// the GPU matched filter of libsa_cuda.so.
#include "sa_finder.h"
#include "sa_matched_filter.h"

extern "C" {

void cleanup(void* flt) { saFilterCleanup(flt); }

void convolve(void* flt, double* image, double* result) { saFilterConvolve(flt, image, result); }

void convolveMemo(void* flt, double* image, double* result) { saFilterConvolveMemo(flt, image, result); }

void* initialize(double* psf, double max_diff, int x_size, int y_size, int estimate) {
  return saFilterCreate(psf, max_diff, x_size, y_size, estimate);
}

}  // extern "C"
