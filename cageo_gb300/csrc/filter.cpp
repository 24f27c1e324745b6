// filter.cpp -- A2 process-convolution filter, host FP64
// (src/convolution/ConvolutionAlgorithm.cpp:18-172, which uses FFTW and
// Eigen; neither is used here).
//
//  1. correlogram over [-r, r]^2 with the reference's float/double mix:
//     exponential  (float) expf(-sqrtf(x^2+y^2) / ((range/3)/cell))       (:56-64)
//     Gaussian     (float) exp(-(x^2+y^2) / pow((range/1.73205080757f)/cell, 2))  (:66-74)
//  2. its 2D DFT (the correlogram is real and even, so the spectrum is
//     real); each coefficient becomes sqrt(|F|)                            (:99-115)
//  3. inverse DFT divided by n^2 = (2r+1)^2, then fftshift                (:117-145)
//  4. Gaussian: the filter matrix is symmetric and numerically rank one;
//     its leading singular pair (u0, s0) is found by power iteration and
//     the taps are u0*sqrt(s0)                                              (:150-172)
// The DFTs are computed directly (separable, O(n^3)); n <= 2*radius+1.
// The sign of u0 is arbitrary (as with Eigen's SVD); both convolution
// passes use the taps, so the sign cancels exactly in the result.
#include <cmath>
#include <vector>
#include "cageo.h"
#include "guard.h"

namespace {

// Separable real-input 2D DFT of an even, real n x n array; returns the
// (real) spectrum.  Uses exact cos tables for the n roots of unity.
std::vector<double> dft2_real_even(const std::vector<double>& a, int n) {
  std::vector<double> c(n * n), s(n * n);
  const double tau = 6.283185307179586476925286766559;
  for (int k = 0; k < n; k++)
    for (int j = 0; j < n; j++) {
      int m = (int)(((long long)k * j) % n);
      c[k * n + j] = std::cos(tau * m / n);
      s[k * n + j] = std::sin(tau * m / n);
    }
  // rows: A1[y][kx] = sum_x a[y][x] e^{-i 2pi kx x/n}
  std::vector<double> re(n * n), im(n * n);
  for (int y = 0; y < n; y++)
    for (int kx = 0; kx < n; kx++) {
      double sr = 0, si = 0;
      for (int x = 0; x < n; x++) {
        sr += a[y * n + x] * c[kx * n + x];
        si -= a[y * n + x] * s[kx * n + x];
      }
      re[y * n + kx] = sr;
      im[y * n + kx] = si;
    }
  std::vector<double> out(n * n);
  for (int ky = 0; ky < n; ky++)
    for (int kx = 0; kx < n; kx++) {
      double sr = 0, si = 0;
      for (int y = 0; y < n; y++) {
        double cr = c[ky * n + y], ci = -s[ky * n + y];
        sr += re[y * n + kx] * cr - im[y * n + kx] * ci;
        si += re[y * n + kx] * ci + im[y * n + kx] * cr;
      }
      // |F| of the complex result; the imaginary part is round-off here.
      out[ky * n + kx] = std::sqrt(sr * sr + si * si);
    }
  return out;
}

// Inverse real DFT of a real, even spectrum (unnormalised, like FFTW c2r).
std::vector<double> idft2_real_even(const std::vector<double>& F, int n) {
  std::vector<double> c(n * n);
  const double tau = 6.283185307179586476925286766559;
  for (int k = 0; k < n; k++)
    for (int j = 0; j < n; j++) c[k * n + j] = std::cos(tau * (double)(((long long)k * j) % n) / n);
  std::vector<double> t(n * n), out(n * n);
  for (int ky = 0; ky < n; ky++)
    for (int x = 0; x < n; x++) {
      double sum = 0;
      for (int kx = 0; kx < n; kx++) sum += F[ky * n + kx] * c[kx * n + x];
      t[ky * n + x] = sum;
    }
  for (int y = 0; y < n; y++)
    for (int x = 0; x < n; x++) {
      double sum = 0;
      for (int ky = 0; ky < n; ky++) sum += t[ky * n + x] * c[ky * n + y];
      out[y * n + x] = sum;
    }
  return out;
}

}  // namespace

extern "C" int cageo_filter_radius(float practical_range, float cell_size) {
  volatile float q = practical_range / cell_size;
  volatile float s = q * 2.5f;
  return (int)std::ceil((float)s);
}

static cageo_status filter_build(int model, float range, float cell, int r, float* h_filter) {
  if (!h_filter || r < 0 || r > 512 || !(range > 0) || !(cell > 0)) {
    cageo::set_error("invalid argument: filter output, radius (0..512), range or cell size");
    return CAGEO_ERR_ARGUMENT;
  }
  if (model != CAGEO_FILTER_GAUSSIAN && model != CAGEO_FILTER_EXPONENTIAL) {
    cageo::set_error("invalid argument: filter model");
    return CAGEO_ERR_ARGUMENT;
  }
  const int n = 2 * r + 1;
  std::vector<double> corr(n * n);
  for (int y = -r, i = 0; y <= r; y++)
    for (int x = -r; x <= r; x++, i++) {
      float v;
      if (model == CAGEO_FILTER_EXPONENTIAL) {
        volatile float d = std::sqrt((float)(x * x + y * y));
        volatile float scale = (range / 3.0f) / cell;
        volatile float arg = -d / scale;
        v = std::exp((float)arg);
      } else {
        volatile float scale = (range / 1.73205080757f) / cell;
        double den = std::pow((double)scale, 2);
        v = (float)std::exp(-(double)(x * x + y * y) / den);
      }
      corr[i] = (double)v;
    }
  std::vector<double> F = dft2_real_even(corr, n);
  for (double& f : F) f = std::sqrt(f);
  std::vector<double> k = idft2_real_even(F, n);
  const double nn = (double)n * n;
  std::vector<float> filt(n * n);
  const int sh = n / 2;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++)
      filt[((j + sh) % n) * n + (i + sh) % n] = (float)(k[j * n + i] / nn);
  if (model == CAGEO_FILTER_EXPONENTIAL) {
    for (int i = 0; i < n * n; i++) h_filter[i] = filt[i];
    return CAGEO_OK;
  }
  // Leading singular pair of the (symmetric) filter matrix by power
  // iteration on K^T K.
  std::vector<double> K(n * n), v(n, 1.0 / std::sqrt((double)n)), w(n), u(n);
  for (int i = 0; i < n * n; i++) K[i] = (double)filt[i];
  double sigma = 0;
  for (int it = 0; it < 500; it++) {
    for (int i = 0; i < n; i++) {
      double s = 0;
      for (int j = 0; j < n; j++) s += K[i * n + j] * v[j];
      u[i] = s;
    }
    for (int j = 0; j < n; j++) {
      double s = 0;
      for (int i = 0; i < n; i++) s += K[i * n + j] * u[i];
      w[j] = s;
    }
    double norm = 0;
    for (double x : w) norm += x * x;
    norm = std::sqrt(norm);
    if (norm == 0) break;
    double diff = 0;
    for (int j = 0; j < n; j++) {
      double nv = w[j] / norm;
      diff += std::fabs(nv - v[j]);
      v[j] = nv;
    }
    sigma = std::sqrt(norm);
    if (diff < 1e-15) break;
  }
  // u0 = K v / sigma
  double unorm = 0;
  for (int i = 0; i < n; i++) {
    double s = 0;
    for (int j = 0; j < n; j++) s += K[i * n + j] * v[j];
    u[i] = s;
    unorm += s * s;
  }
  unorm = std::sqrt(unorm);
  if (!(unorm > 0)) {
    cageo::set_error("invalid argument: the filter has no leading singular vector");
    return CAGEO_ERR_ARGUMENT;
  }
  const double root = std::sqrt(sigma);
  for (int i = 0; i < n; i++) h_filter[i] = (float)(u[i] / unorm * root);
  return CAGEO_OK;
}

extern "C" cageo_status cageo_filter_build(int model, float range, float cell, int r,
                                           float* h_filter) {
  return cageo::guarded("cageo_filter_build",
                        [&] { return filter_build(model, range, cell, r, h_filter); });
}
