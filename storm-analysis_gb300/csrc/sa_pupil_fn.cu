// sa_pupil_fn.cu -- host side of the pupil-function PSF model: the
// reference's pupil_function.c C interface (pfnInitialize, pfnSetPF,
// pfnTranslate, pfnTranslateZ, pfnGetPSF, pfnGetPSFIntensity,
// pfnGetPSFdx / dy / dz, pfnSetPNEN and the six dipole PSFs, pfnGetSize,
// pfnCleanup) and the device tables of the engine's pupil model.
//
// The reference transforms with FFTW (a backward 2D complex DFT).  Here the
// transform is a direct separable DFT (pupil functions are a few tens of
// samples across): the sums over the second index, then over the first.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "sa_device.cuh"
#include "sa_pupil_fn.h"

namespace sa {

namespace {

constexpr double kPi = 3.14159265358979323846;   // the reference's M_PI

// e^{2 pi i k n / N}, the phase reduced mod N first
inline void twiddle(long k, long n, long N, double& re, double& im) {
  const double a = 2.0 * kPi * (double)((k * n) % N) / (double)N;
  re = std::cos(a);
  im = std::sin(a);
}

}  // namespace

void pupil_init(PupilH& p, const double* kx, const double* ky, const double* kz, int n) {
  const size_t nn = (size_t)n * n;
  p.n = n;
  p.kx.resize(nn);
  p.ky.resize(nn);
  p.kz.resize(nn);
  for (size_t i = 0; i < nn; i++) {
    p.kx[i] = 2.0 * kPi * kx[i];
    p.ky[i] = 2.0 * kPi * ky[i];
    p.kz[i] = 2.0 * kPi * kz[i];
  }
  p.pf.assign(2 * nn, 0.0);
  p.ws.assign(2 * nn, 0.0);
}

void pupil_set_pf(PupilH& p, const double* r_pf, const double* c_pf) {
  const int n = p.n;
  const double norm = 1.0 / ((double)n);
  for (int i = 0; i < n; i++)
    for (int k = 0; k < n; k++) {
      const size_t l = (size_t)i * n + k;
      // the sign centres the PSF after the inverse transform
      const double s = ((i + k) % 2 == 0) ? 1.0 : -1.0;
      p.pf[2 * l] = s * r_pf[l] * norm;
      p.pf[2 * l + 1] = s * c_pf[l] * norm;
    }
  p.ws = p.pf;
}

void pupil_translate(PupilH& p, double dx, double dy, double dz, bool z_only) {
  const int n = p.n, m = n / 2, m1 = m + 1;
  std::vector<double> xr(n), xc(n), yr(n), yc(n), zr((size_t)m1 * m1), zc((size_t)m1 * m1);
  // x / y: both multipliers from kx's first column (:455-463)
  for (int i = 0; i < n; i++) {
    double dd = p.kx[(size_t)i * n] * dx;
    xr[i] = std::cos(dd);
    xc[i] = -std::sin(dd);
    dd = p.kx[(size_t)i * n] * dy;
    yr[i] = std::cos(dd);
    yc[i] = -std::sin(dd);
  }
  // z over the pie slice with -dz, mirrored (:475-486)
  for (int i = 0; i <= m; i++)
    for (int j = i; j <= m; j++) {
      const double dd = -p.kz[(size_t)(m - i) * n + (m - j)] * dz;
      zr[(size_t)i * m1 + j] = std::cos(dd);
      zc[(size_t)i * m1 + j] = -std::sin(dd);
      zr[(size_t)j * m1 + i] = zr[(size_t)i * m1 + j];
      zc[(size_t)j * m1 + i] = zc[(size_t)i * m1 + j];
    }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      const size_t l = (size_t)i * n + j, o = (size_t)std::abs(i - m) * m1 + std::abs(j - m);
      double r1, c1;
      if (z_only) {
        r1 = zr[o];
        c1 = zc[o];
      } else {
        const double r2 = xr[i] * yr[j] - xc[i] * yc[j];
        const double c2 = xr[i] * yc[j] + xc[i] * yr[j];
        r1 = r2 * zr[o] - c2 * zc[o];
        c1 = r2 * zc[o] + c2 * zr[o];
      }
      p.ws[2 * l] = r1 * p.pf[2 * l] - c1 * p.pf[2 * l + 1];
      p.ws[2 * l + 1] = r1 * p.pf[2 * l + 1] + c1 * p.pf[2 * l];
    }
}

void pupil_transform(const PupilH& p, int which, const double* dipole, double* r, double* c) {
  const int n = p.n;
  const size_t nn = (size_t)n * n;
  std::vector<double> in(2 * nn), mid(2 * nn), er(nn), ei(nn);
  for (size_t l = 0; l < nn; l++) {
    const double wr = p.ws[2 * l], wc = p.ws[2 * l + 1];
    switch (which) {
      case 1: case 2: case 3: {
        // times -i k (:141-142, :166-167, :191-192)
        const double k = (which == 1) ? p.kx[l] : (which == 2 ? p.ky[l] : p.kz[l]);
        in[2 * l] = wc * k;
        in[2 * l + 1] = -wr * k;
        break;
      }
      case 4:
        in[2 * l] = wr * dipole[l];
        in[2 * l + 1] = wc * dipole[l];
        break;
      default:
        in[2 * l] = wr;
        in[2 * l + 1] = wc;
    }
  }
  for (int a = 0; a < n; a++)
    for (int b = 0; b < n; b++) twiddle(a, b, n, er[(size_t)a * n + b], ei[(size_t)a * n + b]);
  // sums over the second index, then over the first
  for (int i = 0; i < n; i++)
    for (int v = 0; v < n; v++) {
      double sr = 0.0, si = 0.0;
      for (int k = 0; k < n; k++) {
        const double ar = in[2 * ((size_t)i * n + k)], ai = in[2 * ((size_t)i * n + k) + 1];
        const double tr = er[(size_t)k * n + v], ti = ei[(size_t)k * n + v];
        sr += ar * tr - ai * ti;
        si += ar * ti + ai * tr;
      }
      mid[2 * ((size_t)i * n + v)] = sr;
      mid[2 * ((size_t)i * n + v) + 1] = si;
    }
  const double sign = (which == 3) ? -1.0 : 1.0;
  for (int u = 0; u < n; u++)
    for (int v = 0; v < n; v++) {
      double sr = 0.0, si = 0.0;
      for (int i = 0; i < n; i++) {
        const double ar = mid[2 * ((size_t)i * n + v)], ai = mid[2 * ((size_t)i * n + v) + 1];
        const double tr = er[(size_t)i * n + u], ti = ei[(size_t)i * n + u];
        sr += ar * tr - ai * ti;
        si += ar * ti + ai * tr;
      }
      r[(size_t)u * n + v] = sign * sr;
      c[(size_t)u * n + v] = sign * si;
    }
}

bool pupil_rows_separable(const PupilH& p) {
  const int n = p.n;
  for (int i = 0; i < n; i++)
    for (int k = 1; k < n; k++)
      if (p.kx[(size_t)i * n + k] != p.kx[(size_t)i * n]) return false;
  return true;
}

int pupil_tables(const PupilH& p, std::vector<double>& out) {
  const int n = p.n, m = n / 2, m1 = m + 1;
  const PupilLayout L = pupil_layout(n);
  out.assign(L.total, 0.0);
  for (int a = 0; a < n; a++)
    for (int b = 0; b < n; b++) twiddle(a, b, n, out[L.e + 2 * (a * n + b)], out[L.e + 2 * (a * n + b) + 1]);
  std::memcpy(out.data() + L.pf, p.pf.data(), sizeof(double) * p.pf.size());
  for (int i = 0; i < n; i++) out[L.kx + i] = p.kx[(size_t)i * n];
  std::memcpy(out.data() + L.ky, p.ky.data(), sizeof(double) * p.ky.size());
  std::memcpy(out.data() + L.kz, p.kz.data(), sizeof(double) * p.kz.size());
  for (int a = 0; a < m1; a++)
    for (int b = 0; b < m1; b++) {
      const int lo = a < b ? a : b, hi = a < b ? b : a;
      out[L.kzs + a * m1 + b] = p.kz[(size_t)(m - lo) * n + (m - hi)];
    }
  // the pupil function's support: rows and per-row columns with a non-zero value
  int i_lo = n, i_hi = -1;
  for (int i = 0; i < n; i++) {
    int k_lo = n, k_hi = -1;
    for (int k = 0; k < n; k++) {
      const size_t l = (size_t)i * n + k;
      if (p.pf[2 * l] != 0.0 || p.pf[2 * l + 1] != 0.0) {
        if (k < k_lo) k_lo = k;
        k_hi = k;
      }
    }
    if (k_hi < 0) {
      k_lo = 1;
      k_hi = 0;
    } else {
      if (i < i_lo) i_lo = i;
      i_hi = i;
    }
    out[L.rng + 2 * i] = (double)k_lo;
    out[L.rng + 2 * i + 1] = (double)k_hi;
  }
  if (i_hi < 0) {
    i_lo = 1;
    i_hi = 0;
  }
  out[L.band] = (double)i_lo;
  out[L.band + 1] = (double)i_hi;
  return i_hi - i_lo + 1;
}

}  // namespace sa

// ---- the reference's pupil_function.c interface (pupilfn/pupil_function_c.py binds it) ----

extern "C" {

// pfnInitialize pupil_function.c:321-363 (the size must be even:
// pupil_function_c.py:101-103 asserts it).
void* pfnInitialize(double* kx, double* ky, double* kz, int size) {
  if (!kx || !ky || !kz || size < 2 || (size % 2) != 0) return nullptr;
  sa::PupilH* p = new sa::PupilH();
  sa::pupil_init(*p, kx, ky, kz, size);
  return p;
}

// pfnCleanup :42-73.
void pfnCleanup(void* pupil_data) { delete reinterpret_cast<sa::PupilH*>(pupil_data); }

// pfnSetPF :370-410.
void pfnSetPF(void* pupil_data, double* r_pf, double* c_pf) {
  sa::pupil_set_pf(*reinterpret_cast<sa::PupilH*>(pupil_data), r_pf, c_pf);
}

// pfnSetPNEN :419-439.
void pfnSetPNEN(void* pupil_data, double* px_ex, double* px_ey, double* py_ex, double* py_ey, double* pz_ex,
                double* pz_ey) {
  sa::PupilH* p = reinterpret_cast<sa::PupilH*>(pupil_data);
  const double* src[6] = {px_ex, px_ey, py_ex, py_ey, pz_ex, pz_ey};
  const size_t nn = (size_t)p->n * p->n;
  for (int i = 0; i < 6; i++) p->pnen[i].assign(src[i], src[i] + nn);
}

// pfnTranslate :448-506, pfnTranslateZ :515-556.
void pfnTranslate(void* pupil_data, double dx, double dy, double dz) {
  sa::pupil_translate(*reinterpret_cast<sa::PupilH*>(pupil_data), dx, dy, dz, false);
}
void pfnTranslateZ(void* pupil_data, double dz) {
  sa::pupil_translate(*reinterpret_cast<sa::PupilH*>(pupil_data), 0.0, 0.0, dz, true);
}

// pfnGetPSF :80-98, pfnGetPSFdx / dy / dz :135-203.
void pfnGetPSF(void* pupil_data, double* r, double* c) {
  sa::pupil_transform(*reinterpret_cast<sa::PupilH*>(pupil_data), 0, nullptr, r, c);
}
void pfnGetPSFdx(void* pupil_data, double* r, double* c) {
  sa::pupil_transform(*reinterpret_cast<sa::PupilH*>(pupil_data), 1, nullptr, r, c);
}
void pfnGetPSFdy(void* pupil_data, double* r, double* c) {
  sa::pupil_transform(*reinterpret_cast<sa::PupilH*>(pupil_data), 2, nullptr, r, c);
}
void pfnGetPSFdz(void* pupil_data, double* r, double* c) {
  sa::pupil_transform(*reinterpret_cast<sa::PupilH*>(pupil_data), 3, nullptr, r, c);
}

// pfnGetPSFIntensity :108-128.
void pfnGetPSFIntensity(void* pupil_data, double* psf) {
  sa::PupilH* p = reinterpret_cast<sa::PupilH*>(pupil_data);
  const size_t nn = (size_t)p->n * p->n;
  std::vector<double> r(nn), c(nn);
  sa::pupil_transform(*p, 0, nullptr, r.data(), c.data());
  for (size_t i = 0; i < nn; i++) psf[i] = r[i] * r[i] + c[i] * c[i];
}

// pfnGetPXEX .. pfnGetPZEY :239-302 (pfnGetPNEN :212-230 with each dipole
// pattern; the patterns must have been set).
static void get_pnen(void* pupil_data, int which, double* r, double* c) {
  sa::PupilH* p = reinterpret_cast<sa::PupilH*>(pupil_data);
  if (p->pnen[which].empty()) return;
  sa::pupil_transform(*p, 4, p->pnen[which].data(), r, c);
}
void pfnGetPXEX(void* pupil_data, double* r, double* c) { get_pnen(pupil_data, 0, r, c); }
void pfnGetPXEY(void* pupil_data, double* r, double* c) { get_pnen(pupil_data, 1, r, c); }
void pfnGetPYEX(void* pupil_data, double* r, double* c) { get_pnen(pupil_data, 2, r, c); }
void pfnGetPYEY(void* pupil_data, double* r, double* c) { get_pnen(pupil_data, 3, r, c); }
void pfnGetPZEX(void* pupil_data, double* r, double* c) { get_pnen(pupil_data, 4, r, c); }
void pfnGetPZEY(void* pupil_data, double* r, double* c) { get_pnen(pupil_data, 5, r, c); }

// pfnGetSize :309-312.
int pfnGetSize(void* pupil_data) { return reinterpret_cast<sa::PupilH*>(pupil_data)->n; }

}  // extern "C"
