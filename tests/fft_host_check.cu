// Host-side check of the Stockham line transform of msx_fft.cuh: every
// schedule's index arithmetic, twiddle tables and register codelets are run
// on the CPU (one emulated thread at a time) and compared with a direct DFT
// evaluated in double precision.  Prints one line per schedule and exits
// non-zero when a relative L2 error exceeds 5e-7.
#include "msx_fft.cuh"
#include "msx_tma.cuh"
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
// The exchange of PairedFFT512: every half warp's store of one register and
// every half warp's load of one element touch sixteen distinct bank pairs
// (a float2 spans two 4-byte banks), and the swizzle is a permutation.
bool paired_banks_ok() {
  using P = PairedFFT512;
  auto sw = [](int i) { return i ^ ((i >> 5) & 15); };
  bool seen[512] = {};
  for (int i = 0; i < 512; ++i) {
    if (seen[sw(i)]) return false;
    seen[sw(i)] = true;
  }
  for (int m = 0; m < 16; ++m)
    for (int half = 0; half < 2; ++half) {
      bool st[16] = {}, ld[16] = {};
      for (int l = 0; l < 16; ++l) {
        const int t = 16 * half + l;
        const int bs = sw(P::pos(m, t)) & 15, bl = sw(t + 32 * m) & 15;
        if (st[bs] || ld[bl]) return false;
        st[bs] = ld[bl] = true;
      }
    }
  // the byte-offset forms of the device code: for a 256-byte-aligned line L,
  // (L + st_base(t)) ^ 8 c_m and ((L + 8 t) ^ 8 m) + 256 m address the same
  // words as the swizzled indices
  for (unsigned L : {0u, 256u, 0x9100u, 0x2a700u})
    for (int t = 0; t < 32; ++t)
      for (int m = 0; m < 16; ++m) {
        const unsigned cm = 8u * (m + (m >= 8 ? 8 : 0));
        if (P::st_off(m, t) != 8u * sw(P::pos(m, t)) || P::ld_off(m, t) != 8u * sw(t + 32 * m)) return false;
        if (((L + P::st_base(t)) ^ cm) != L + P::st_off(m, t)) return false;
        if ((((L + 8u * t) ^ (8u * m)) + 256u * m) != L + P::ld_off(m, t)) return false;
      }
  // every position is written exactly once
  bool hit[512] = {};
  for (int t = 0; t < 32; ++t)
    for (int m = 0; m < 16; ++m) {
      if (hit[P::pos(m, t)]) return false;
      hit[P::pos(m, t)] = true;
    }
  return true;
}
// The column pass's tile order visits every (wave, column tile) of the range
// exactly once, and the two tiles of each aligned pair inside the range
// consecutively.
bool col_tile_order_ok() {
  for (int G : {1, 2, 3, 7, 64})
    for (int xt0 = 0; xt0 < 9; ++xt0)
      for (int tx = 1; tx < 14; ++tx) {
        std::vector<char> seen(G * tx, 0);
        int prev_p = -1, prev_xt = -1;
        for (int u = 0; u < G * tx; ++u) {
          int p = -1, xt = -1;
          col_tile_order(u, G, xt0, tx, p, xt);
          if (p < 0 || p >= G || xt < xt0 || xt >= xt0 + tx) return false;
          char& s = seen[p * tx + (xt - xt0)];
          if (s) return false;
          s = 1;
          // an odd tile whose even partner is in the range follows it directly
          if ((xt & 1) && xt - 1 >= xt0 && (prev_p != p || prev_xt != xt - 1)) return false;
          prev_p = p; prev_xt = xt;
        }
      }
  return true;
}
int main() {
  double w = 0;
  const bool order = col_tile_order_ok();
  printf("column tile order: %s\n", order ? "yes" : "NO");
  if (!order) return 1;
  const bool banks = paired_banks_ok();
  printf("paired exchange conflict-free: %s\n", banks ? "yes" : "NO");
  if (!banks) return 1;
  w = fmax(w, check<LineFFT<64, 8, Radices<8, 8>>, 64>());
  w = fmax(w, check<LineFFT<128, 8, Radices<16, 8>>, 128>());
  w = fmax(w, check<LineFFT<256, 16, Radices<16, 16>>, 256>());
  w = fmax(w, check<LineFFT<256, 32, Radices<8, 8, 4>>, 256>());
  w = fmax(w, check<LineFFT<384, 16, Radices<8, 8, 6>>, 384>());
  w = fmax(w, check<LineFFT<512, 16, Radices<32, 16>>, 512>());
  w = fmax(w, check<LineFFT<512, 32, Radices<16, 16, 2>>, 512>());
  w = fmax(w, check<LineFFT<512, 32, Radices<8, 8, 8>>, 512>());
  w = fmax(w, check<LineFFT<512, 32, Radices<16, 2, 16>>, 512>());
  w = fmax(w, check<PairedFFT512, 512>());
  w = fmax(w, check<LineFFT<768, 32, Radices<8, 8, 12>>, 768>());
  w = fmax(w, check<LineFFT<1024, 32, Radices<32, 32>>, 1024>());
  w = fmax(w, check<LineFFT<1024, 32, Radices<16, 8, 8>>, 1024>());
  return w < 5e-7 ? 0 : 1;
}
