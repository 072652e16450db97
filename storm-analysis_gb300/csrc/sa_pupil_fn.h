// sa_pupil_fn.h -- the pupil function of the reference's pupil_function.c
// on the host: its translation (pfnTranslate), the complex PSF and its
// derivatives (pfnGetPSF*), and the table set the engine's pupil-function
// model reads on the device.
#pragma once

#include <vector>

namespace sa {

// A pupil function of n x n samples (n even), with the geometry's
// translation multipliers (2 pi kx, 2 pi ky, 2 pi kz), the pupil function as
// pfnSetPF stores it (divided by n, negated where i + k is odd) and the
// working copy of the current translation, all (re, im) for the complex ones.
struct PupilH {
  int n = 0;
  std::vector<double> kx, ky, kz;
  std::vector<double> pf, ws;
  std::vector<double> pnen[6];   // dipole patterns (pfnSetPNEN), empty until set
};

// pfnInitialize pupil_function.c:321-363 (the pupil function starts at 0).
void pupil_init(PupilH& p, const double* kx, const double* ky, const double* kz, int n);

// pfnSetPF :370-410.
void pupil_set_pf(PupilH& p, const double* r_pf, const double* c_pf);

// pfnTranslate :448-506 (z_only: pfnTranslateZ :515-556).
void pupil_translate(PupilH& p, double dx, double dy, double dz, bool z_only);

// FFTW's unnormalised backward 2D transform of the working pupil function
// times a factor per element: which 0 none (pfnGetPSF), 1 / 2 / 3 -i kx,
// -i ky, -i kz (pfnGetPSFdx / dy / dz; dz negated as :199-201), 4 a real
// dipole pattern (pfnGetPNEN :212-230).  Outputs n x n (re) and (im).
void pupil_transform(const PupilH& p, int which, const double* dipole, double* r, double* c);

// True when kx is constant along the pupil's rows (the engine's x
// derivative takes kx per row, as pfnTranslate takes the x shift).
bool pupil_rows_separable(const PupilH& p);

// The device tables of the engine's pupil model (pupil_layout in
// sa_device.cuh).  Returns the rows of the pupil's support band (0 if the
// pupil function is zero everywhere).
int pupil_tables(const PupilH& p, std::vector<double>& out);

}  // namespace sa
