// sa_ia_utilities.cpp -- libsa_ia_utilities.so: the reference-named
// image-analysis utilities (include/sa_ia_utilities.h), forwarding to the GPU
// implementations in libsa_cuda.so.
#include "sa_ia_utilities.h"

extern "C" {

int calcMaxPeaks(saFlmData* flm_data) { return saCalcMaxPeaks(flm_data); }

void* createKDTree(double* x, double* y, int n) { return saCreateKDTree(x, y, n); }

void findLocalMaxima(saFlmData* flm_data, double* z, double* y, double* x, double* h) {
  saFindLocalMaxima(flm_data, z, y, x, h);
}

void freeKDTree(void* kd) { saFreeKDTree(kd); }

int markDimmerPeaks(double* x, double* y, double* h, int32_t* status, double r_removal, double r_neighbors, int np) {
  return saMarkDimmerPeaks(x, y, h, status, r_removal, r_neighbors, np);
}

int markLowSignificancePeaks(double* x, double* y, double* sig, int32_t* status, double min_sig, double r_neighbors,
                             int np) {
  return saMarkLowSignificancePeaks(x, y, sig, status, min_sig, r_neighbors, np);
}

void nearestKDTree(void* kd, double* x, double* y, double* dist, int32_t* index, double radius, int n) {
  saNearestKDTree(kd, x, y, dist, index, radius, n);
}

void runningIfHasNeighbors(double* c_x, double* c_y, double* n_x, double* n_y, int32_t* status, double radius,
                           int nc, int nn) {
  saRunningIfHasNeighbors(c_x, c_y, n_x, n_y, status, radius, nc, nn);
}

}  // extern "C"
