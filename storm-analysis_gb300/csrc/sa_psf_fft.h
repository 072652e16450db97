// sa_psf_fft.h -- the FFT-translated 3D PSF of the reference's psf_fft.c on
// the host: the PSF's spectrum (pFTInitialize), the translated middle-plane
// PSF and its derivatives (pFTTranslate / pFTGetPSF*), and the table set the
// engine's FFT PSF model reads on the device.
#pragma once

#include <vector>

namespace sa {

// A PSF of nz x ny x nx samples (x fastest), with its r2c spectrum
// (nz x ny x (nx/2 + 1) complex, as (re, im)) and the current translation's
// shift vectors.
struct PsfFFTH {
  int nz = 0, ny = 0, nx = 0;
  std::vector<double> spec;
  double dx = 0.0, dy = 0.0, dz = 0.0;
};

// pFTInitialize psf_fft.c:310-365: the spectrum of psf / (nz ny nx).
void psf_fft_init(PsfFFTH& p, const double* psf, int nz, int ny, int nx);

// The middle z plane of the c2r inverse of the translated spectrum
// (which 0: the PSF, 1-3: its x, y, z derivatives as pFTGetPSFdx / dy / dz),
// ny x nx values.
void psf_fft_plane(const PsfFFTH& p, int which, double* out);

// The device tables of the engine's FFT model (fft_layout in sa_device.cuh).
void psf_fft_tables(const PsfFFTH& p, std::vector<double>& out);

}  // namespace sa
