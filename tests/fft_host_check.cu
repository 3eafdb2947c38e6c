// Host-side check of the Stockham line transform of msx_fft.cuh: every
// schedule's index arithmetic, twiddle tables and register codelets are run
// on the CPU (one emulated thread at a time) and compared with a direct DFT
// evaluated in double precision.  Prints one line per schedule and exits
// non-zero when a relative L2 error exceeds 5e-7.
#include "msx_fft.cuh"
#include <cstdio>
#include <cmath>
#include <vector>
#include <random>
using namespace msx;
template <class F, int N> double check() {
  std::vector<float2> tw(F::tw_words() + 1);
  F::host_twiddles(tw.data());
  std::mt19937 rng(1); std::uniform_real_distribution<float> U(-1, 1);
  std::vector<float2> x(N), y(N);
  for (auto& e : x) e = make_float2(U(rng), U(rng));
  double worst = 0;
  for (int inv = 0; inv < 2; ++inv) {
    y = x;
    if (inv) F::template host_run<true>(y.data(), tw.data()); else F::template host_run<false>(y.data(), tw.data());
    double num = 0, den = 0;
    for (int k = 0; k < N; ++k) {
      double re = 0, im = 0;
      for (int n = 0; n < N; ++n) {
        double a = (inv ? 2 : -2) * M_PI * double((long)n * k % N) / N;
        re += x[n].x * cos(a) - x[n].y * sin(a);
        im += x[n].x * sin(a) + x[n].y * cos(a);
      }
      num += (y[k].x - re) * (y[k].x - re) + (y[k].y - im) * (y[k].y - im);
      den += re * re + im * im;
    }
    worst = fmax(worst, sqrt(num / den));
  }
  printf("N=%4d T=%2d E=%2d rel err %.3e\n", N, N / F::E, F::E, worst);
  return worst;
}
int main() {
  double w = 0;
  w = fmax(w, check<LineFFT<64, 8, Radices<8, 8>>, 64>());
  w = fmax(w, check<LineFFT<128, 8, Radices<16, 8>>, 128>());
  w = fmax(w, check<LineFFT<256, 16, Radices<16, 16>>, 256>());
  w = fmax(w, check<LineFFT<256, 32, Radices<8, 8, 4>>, 256>());
  w = fmax(w, check<LineFFT<384, 16, Radices<8, 8, 6>>, 384>());
  w = fmax(w, check<LineFFT<512, 16, Radices<32, 16>>, 512>());
  w = fmax(w, check<LineFFT<512, 32, Radices<16, 16, 2>>, 512>());
  w = fmax(w, check<LineFFT<512, 32, Radices<8, 8, 8>>, 512>());
  w = fmax(w, check<LineFFT<512, 32, Radices<16, 2, 16>>, 512>());
  w = fmax(w, check<LineFFT<768, 32, Radices<8, 8, 12>>, 768>());
  w = fmax(w, check<LineFFT<1024, 32, Radices<32, 32>>, 1024>());
  w = fmax(w, check<LineFFT<1024, 32, Radices<16, 8, 8>>, 1024>());
  return w < 5e-7 ? 0 : 1;
}
