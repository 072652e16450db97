// sa_psf_fft.cu -- host side of the FFT PSF model: the reference's psf_fft.c
// C interface (pFTInitialize, pFTTranslate, pFTGetPSF, pFTGetPSFdx / dy / dz,
// pFTGetX/Y/ZSize, pFTCleanup) and the device tables of the engine's FFT
// PSF model.
//
// The reference transforms with FFTW.  Here the transforms are direct
// separable DFT sums (PSFs are a few tens of samples per axis): the forward
// r2c transform once per PSF, and for a translated PSF only its middle z
// plane -- the only plane the reference reads (psf_fft.c:131-136) -- as the
// c2r inverse would give it (complex inverses along z and y, then the c2r
// along x, which drops the imaginary parts of the x DC and Nyquist bins).
#include <cmath>
#include <cstring>
#include <vector>

#include "sa_device.cuh"
#include "sa_psf_fft.h"

namespace sa {

namespace {

constexpr double kPi = 3.14159265358979323846;   // the reference's M_PI

// e^{sign 2 pi i k n / N}, the phase reduced mod N first
inline void twiddle(long k, long n, long N, int sign, double& re, double& im) {
  const double a = 2.0 * kPi * (double)((k * n) % N) / (double)N;
  re = std::cos(a);
  im = sign * std::sin(a);
}

// pFTCalcShiftVector psf_fft.c:43-60 (entry size/2 keeps the positive sine).
void shift_vector(double d, int size, std::vector<double>& re, std::vector<double>& im) {
  re.assign(size, 0.0);
  im.assign(size, 0.0);
  re[0] = 1.0;
  const double t1 = -kPi * 2.0 * d / ((double)size);
  for (int i = 1; i < (size / 2 + 1); i++) {
    const double t2 = t1 * (double)i;
    const double tr = std::cos(t2), tc = std::sin(t2);
    re[size - i] = tr;
    re[i] = tr;
    im[size - i] = -tc;
    im[i] = tc;
  }
}

// pFTCalcShiftVectorDerivative psf_fft.c:70-84.
void shift_derivative(int size, std::vector<double>& d) {
  d.assign(size, 0.0);
  const double t1 = -kPi * 2.0 / ((double)size);
  for (int i = 1; i < (size / 2 + 1); i++) {
    const double t2 = t1 * (double)i;
    d[size - i] = t2;
    d[i] = -t2;
  }
}

}  // namespace

void psf_fft_init(PsfFFTH& p, const double* psf, int nz, int ny, int nx) {
  p.nz = nz;
  p.ny = ny;
  p.nx = nx;
  const int nk = nx / 2 + 1;
  const double norm = 1.0 / ((double)nz * ny * nx);
  // along x (r2c), then y, then z
  std::vector<double> ax((size_t)nz * ny * nk * 2, 0.0);
  for (int z = 0; z < nz; z++)
    for (int y = 0; y < ny; y++)
      for (int kx = 0; kx < nk; kx++) {
        double sr = 0.0, si = 0.0;
        for (int x = 0; x < nx; x++) {
          double er, ei;
          twiddle(kx, x, nx, -1, er, ei);
          const double v = psf[((size_t)z * ny + y) * nx + x] * norm;
          sr += v * er;
          si += v * ei;
        }
        double* o = &ax[2 * (((size_t)z * ny + y) * nk + kx)];
        o[0] = sr;
        o[1] = si;
      }
  std::vector<double> axy(ax.size(), 0.0);
  for (int z = 0; z < nz; z++)
    for (int ky = 0; ky < ny; ky++)
      for (int kx = 0; kx < nk; kx++) {
        double sr = 0.0, si = 0.0;
        for (int y = 0; y < ny; y++) {
          double er, ei;
          twiddle(ky, y, ny, -1, er, ei);
          const double* a = &ax[2 * (((size_t)z * ny + y) * nk + kx)];
          sr += a[0] * er - a[1] * ei;
          si += a[0] * ei + a[1] * er;
        }
        double* o = &axy[2 * (((size_t)z * ny + ky) * nk + kx)];
        o[0] = sr;
        o[1] = si;
      }
  p.spec.assign(ax.size(), 0.0);
  for (int kz = 0; kz < nz; kz++)
    for (int ky = 0; ky < ny; ky++)
      for (int kx = 0; kx < nk; kx++) {
        double sr = 0.0, si = 0.0;
        for (int z = 0; z < nz; z++) {
          double er, ei;
          twiddle(kz, z, nz, -1, er, ei);
          const double* a = &axy[2 * (((size_t)z * ny + ky) * nk + kx)];
          sr += a[0] * er - a[1] * ei;
          si += a[0] * ei + a[1] * er;
        }
        double* o = &p.spec[2 * (((size_t)kz * ny + ky) * nk + kx)];
        o[0] = sr;
        o[1] = si;
      }
  p.dx = p.dy = p.dz = 0.0;
}

void psf_fft_plane(const PsfFFTH& p, int which, double* out) {
  const int nx = p.nx, ny = p.ny, nz = p.nz, nk = nx / 2 + 1, zm = nz / 2;
  std::vector<double> sxr, sxi, syr, syi, szr, szi, dkx, dky, dkz;
  shift_vector(p.dx, nx, sxr, sxi);
  shift_vector(p.dy, ny, syr, syi);
  shift_vector(-p.dz, nz, szr, szi);   // pFTTranslate psf_fft.c:388-391
  shift_derivative(nx, dkx);
  shift_derivative(ny, dky);
  shift_derivative(nz, dkz);
  std::vector<double> C((size_t)ny * nk * 2, 0.0);
  for (int ky = 0; ky < ny; ky++)
    for (int kx = 0; kx < nk; kx++) {
      double cr = 0.0, ci = 0.0;
      for (int kz = 0; kz < nz; kz++) {
        const double* w = &p.spec[2 * (((size_t)kz * ny + ky) * nk + kx)];
        double r1 = w[0], c1 = w[1], r2, c2;
        r2 = r1 * szr[kz] - c1 * szi[kz];
        c2 = r1 * szi[kz] + c1 * szr[kz];
        r1 = r2 * syr[ky] - c2 * syi[ky];
        c1 = r2 * syi[ky] + c2 * syr[ky];
        r2 = r1 * sxr[kx] - c1 * sxi[kx];
        c2 = r1 * sxi[kx] + c1 * sxr[kx];
        if (which == 3) {   // times -i dkz
          const double t = r2;
          r2 = c2 * dkz[kz];
          c2 = -t * dkz[kz];
        }
        double er, ei;
        twiddle(kz, zm, nz, 1, er, ei);
        cr += r2 * er - c2 * ei;
        ci += r2 * ei + c2 * er;
      }
      C[2 * (ky * nk + kx)] = cr;
      C[2 * (ky * nk + kx) + 1] = ci;
    }
  std::vector<double> D((size_t)ny * nk * 2, 0.0);
  for (int y = 0; y < ny; y++)
    for (int kx = 0; kx < nk; kx++) {
      double dr = 0.0, di = 0.0;
      for (int ky = 0; ky < ny; ky++) {
        double ar = C[2 * (ky * nk + kx)], ai = C[2 * (ky * nk + kx) + 1];
        if (which == 2) {   // times -i dky
          const double t = ar;
          ar = ai * dky[ky];
          ai = -t * dky[ky];
        }
        double er, ei;
        twiddle(ky, y, ny, 1, er, ei);
        dr += ar * er - ai * ei;
        di += ar * ei + ai * er;
      }
      D[2 * (y * nk + kx)] = dr;
      D[2 * (y * nk + kx) + 1] = di;
    }
  for (int y = 0; y < ny; y++)
    for (int x = 0; x < nx; x++) {
      double v = 0.0;
      for (int kx = 0; kx < nk; kx++) {
        double ar = D[2 * (y * nk + kx)], ai = D[2 * (y * nk + kx) + 1];
        if (which == 1) {   // times -i dkx
          const double t = ar;
          ar = ai * dkx[kx];
          ai = -t * dkx[kx];
        }
        double er, ei;
        twiddle(kx, x, nx, 1, er, ei);
        const double c = ((kx == 0) || (2 * kx == nx)) ? 1.0 : 2.0;
        v += c * (ar * er - ai * ei);
      }
      out[(size_t)y * nx + x] = (which == 3) ? -v : v;
    }
}

void psf_fft_tables(const PsfFFTH& p, std::vector<double>& out) {
  const int nx = p.nx, ny = p.ny, nz = p.nz;
  const FFTLayout L = fft_layout(nx, ny, nz);
  out.assign(L.total, 0.0);
  std::memcpy(out.data() + L.w, p.spec.data(), sizeof(double) * p.spec.size());
  for (int x = 0; x < nx; x++)
    for (int kx = 0; kx < L.nk; kx++) twiddle(kx, x, nx, 1, out[L.ex + 2 * (x * L.nk + kx)], out[L.ex + 2 * (x * L.nk + kx) + 1]);
  for (int y = 0; y < ny; y++)
    for (int ky = 0; ky < ny; ky++) twiddle(ky, y, ny, 1, out[L.ey + 2 * (y * ny + ky)], out[L.ey + 2 * (y * ny + ky) + 1]);
  for (int kz = 0; kz < nz; kz++) twiddle(kz, nz / 2, nz, 1, out[L.ez + 2 * kz], out[L.ez + 2 * kz + 1]);
  std::vector<double> d;
  shift_derivative(nx, d);
  for (int k = 0; k < L.nk; k++) out[L.dkx + k] = d[k];
  shift_derivative(ny, d);
  for (int k = 0; k < ny; k++) out[L.dky + k] = d[k];
  shift_derivative(nz, d);
  for (int k = 0; k < nz; k++) out[L.dkz + k] = d[k];
}

}  // namespace sa

// ---- the reference's psf_fft.c interface (psf_fft/psf_fft_c.py binds it) ----

extern "C" {

// pFTInitialize psf_fft.c:310-365.
void* pFTInitialize(double* psf, int z_size, int y_size, int x_size) {
  if (!psf || z_size < 1 || y_size < 2 || x_size < 2) return nullptr;
  sa::PsfFFTH* p = new sa::PsfFFTH();
  sa::psf_fft_init(*p, psf, z_size, y_size, x_size);
  return p;
}

// pFTCleanup psf_fft.c:89-106.
void pFTCleanup(void* pfft) { delete reinterpret_cast<sa::PsfFFTH*>(pfft); }

// pFTTranslate psf_fft.c:372-420.
void pFTTranslate(void* pfft, double dx, double dy, double dz) {
  sa::PsfFFTH* p = reinterpret_cast<sa::PsfFFTH*>(pfft);
  if (!p) return;
  p->dx = dx;
  p->dy = dy;
  p->dz = dz;
}

// pFTGetPSF psf_fft.c:116-137, pFTGetPSFdx / dy / dz :147-272.
void pFTGetPSF(void* pfft, double* psf) { sa::psf_fft_plane(*reinterpret_cast<sa::PsfFFTH*>(pfft), 0, psf); }
void pFTGetPSFdx(void* pfft, double* dx) { sa::psf_fft_plane(*reinterpret_cast<sa::PsfFFTH*>(pfft), 1, dx); }
void pFTGetPSFdy(void* pfft, double* dy) { sa::psf_fft_plane(*reinterpret_cast<sa::PsfFFTH*>(pfft), 2, dy); }
void pFTGetPSFdz(void* pfft, double* dz) { sa::psf_fft_plane(*reinterpret_cast<sa::PsfFFTH*>(pfft), 3, dz); }

// pFTGetXSize / YSize / ZSize psf_fft.c:274-296.
int pFTGetXSize(void* pfft) { return reinterpret_cast<sa::PsfFFTH*>(pfft)->nx; }
int pFTGetYSize(void* pfft) { return reinterpret_cast<sa::PsfFFTH*>(pfft)->ny; }
int pFTGetZSize(void* pfft) { return reinterpret_cast<sa::PsfFFTH*>(pfft)->nz; }

}  // extern "C"
