// Register/shared-memory FFT building blocks for the multislice passes.
//
// A "line" is one row or one column of a wave (length N).  T threads share a
// line and each holds E = N/T complex values; thread t always holds the
// elements with index t + T*m (m = 0..E-1), in natural order.  A line
// transform is a sequence of Stockham stages (radices R1*R2*...*Rs = N, each
// Ri dividing E).  Stage i performs E/Ri radix-Ri butterflies per thread in
// registers; between stages the values are exchanged through shared memory.
// Because the Stockham output of the last stage lands in exactly the slots the
// first stage reads, a transform with s stages costs s-1 exchanges and no
// bit-reversal pass, and a forward transform can follow an inverse one (or a
// point-wise multiply) directly in registers.
//
// Twiddles inside a butterfly are compile-time constants (cos/sin of 2*pi*m/R
// evaluated by constexpr Taylor series after exact octant reduction); the
// inter-stage twiddles W_{Ns*R}^{k*r} come from a per-plan table computed in
// double precision on the host and staged into shared memory.
#pragma once
#include <cuda_runtime.h>
#include <utility>

namespace msx {

// ----------------------------------------------------------------- complex helpers
// On the device, componentwise complex additions and scalings use the packed
// two-lane FP32 instructions (add/sub/fma.rn.f32x2): two IEEE operations, the
// same results as the scalar forms, in one issue slot.
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ unsigned long long pk(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 upk(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk(a)), "l"(pk(b)));
  return upk(r);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk(a)), "l"(pk(b)));
  return upk(r);
}
// a + s b (s a scalar)
__device__ __forceinline__ float2 caxpy(float s, float2 b, float2 a) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pk(make_float2(s, s))), "l"(pk(b)), "l"(pk(a)));
  return upk(r);
}
#else
__host__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __forceinline__ float2 caxpy(float s, float2 b, float2 a) {
  return make_float2(fmaf(s, b.x, a.x), fmaf(s, b.y, a.y));
}
#endif
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// ----------------------------------------------------------------- constexpr trig
// sin and cos of x for |x| <= pi/4 by Taylor series (terms to x^25: error far
// below double rounding).
__host__ __device__ constexpr double ce_sin_small(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int n = 1; n < 13; ++n) { term *= -x2 / double((2 * n) * (2 * n + 1)); sum += term; }
  return sum;
}
__host__ __device__ constexpr double ce_cos_small(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int n = 1; n < 13; ++n) { term *= -x2 / double((2 * n - 1) * (2 * n)); sum += term; }
  return sum;
}
constexpr double kHalfPi = 1.57079632679489661923132169163975144;
// cos(2*pi*m/R) (want_sin = false) or sin(2*pi*m/R) (want_sin = true).
// The angle is split exactly into a quadrant and a remainder in [0, pi/4].
__host__ __device__ constexpr double ce_trig2pi(long m, long R, bool want_sin) {
  long a = ((m % R) + R) % R;
  long q = (4 * a) / R;            // quadrant 0..3
  long rem = 4 * a - q * R;        // angle within quadrant = (pi/2)*rem/R
  double c = 0, s = 0;
  if (2 * rem <= R) {
    double phi = kHalfPi * double(rem) / double(R);
    c = ce_cos_small(phi); s = ce_sin_small(phi);
  } else {
    double psi = kHalfPi * double(R - rem) / double(R);
    c = ce_sin_small(psi); s = ce_cos_small(psi);
  }
  double cq = c, sq = s;
  if (q == 1) { cq = -s; sq = c; }
  else if (q == 2) { cq = -c; sq = -s; }
  else if (q == 3) { cq = s; sq = -c; }
  return want_sin ? sq : cq;
}

// v * exp(sign * 2*pi*i * M / R), sign = -1 forward, +1 inverse, M a compile-time constant.
template <int R, int M, bool INV>
__host__ __device__ __forceinline__ float2 twc(float2 v) {
  constexpr int m = ((M % R) + R) % R;
  if constexpr (m == 0) {
    return v;
  } else if constexpr (2 * m == R) {
    return make_float2(-v.x, -v.y);
  } else if constexpr (4 * m == R) {           // fwd: -i   inv: +i
    return INV ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
  } else if constexpr (4 * m == 3 * R) {       // fwd: +i   inv: -i
    return INV ? make_float2(v.y, -v.x) : make_float2(-v.y, v.x);
  } else if constexpr ((8 * m) % R == 0) {     // odd multiples of pi/4
    constexpr float h = 0.70710678118654752440f;
    constexpr int o = (8 * m) / R;             // 1, 3, 5, 7
    // e^{-i pi o/4} (fwd) = (cx + i sx)/sqrt2 with the signs below
    constexpr float cx = (o == 1 || o == 7) ? 1.f : -1.f;
    constexpr float sxf = (o == 1 || o == 3) ? -1.f : 1.f;  // sign of sin for forward
    constexpr float sx = INV ? -sxf : sxf;
    // (a + ib)(cx + i sx) = (a cx - b sx) + i (a sx + b cx)
    return make_float2(h * (cx * v.x - sx * v.y), h * (sx * v.x + cx * v.y));
  } else {
    constexpr float c = (float)ce_trig2pi(m, R, false);
    constexpr float s = (INV ? 1.f : -1.f) * (float)ce_trig2pi(m, R, true);
    return make_float2(fmaf(v.x, c, -v.y * s), fmaf(v.x, s, v.y * c));
  }
}

// ----------------------------------------------------------------- register DFT codelets
template <int R, bool INV> struct Dft;

template <bool INV> struct Dft<1, INV> {
  static __host__ __device__ __forceinline__ void run(float2 (&)[1]) {}
};

template <bool INV> struct Dft<2, INV> {
  static __host__ __device__ __forceinline__ void run(float2 (&v)[2]) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool INV> struct Dft<3, INV> {
  static __host__ __device__ __forceinline__ void run(float2 (&v)[3]) {
    constexpr float s3 = 0.86602540378443864676f;  // sin(2 pi / 3)
    float2 t1 = cadd(v[1], v[2]);
    float2 t2 = make_float2(fmaf(-0.5f, t1.x, v[0].x), fmaf(-0.5f, t1.y, v[0].y));
    float2 h = cscale(csub(v[1], v[2]), s3);
    v[0] = cadd(v[0], t1);
    // forward: X1 = t2 - i h, X2 = t2 + i h
    float2 m1 = make_float2(t2.x + h.y, t2.y - h.x);
    float2 m2 = make_float2(t2.x - h.y, t2.y + h.x);
    v[1] = INV ? m2 : m1;
    v[2] = INV ? m1 : m2;
  }
};

template <bool INV> struct Dft<4, INV> {
  static __host__ __device__ __forceinline__ void run(float2 (&v)[4]) {
    float2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    float2 c = cadd(v[1], v[3]), d = csub(v[1], v[3]);
    // -i d = (d.y, -d.x); +i d = (-d.y, d.x)
    float2 jd = INV ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
    v[0] = cadd(a, c);
    v[2] = csub(a, c);
    v[1] = cadd(b, jd);
    v[3] = csub(b, jd);
  }
};

// Composite DFT of size A*B by one Cooley-Tukey step in registers:
// X[ka + A*kb] = sum_b W_B^{b kb} W_{AB}^{b ka} sum_a x[b + B a] W_A^{a ka}.
template <int A, int B, bool INV, int b, int... ka>
__host__ __device__ __forceinline__ void ct_twiddle(float2 (&u)[A], float2 (&tmp)[A * B], std::integer_sequence<int, ka...>) {
  ((tmp[b + B * ka] = twc<A * B, b * ka, INV>(u[ka])), ...);
}
template <int A, int B, bool INV, int b>
__host__ __device__ __forceinline__ void ct_first(float2 (&v)[A * B], float2 (&tmp)[A * B]) {
  float2 u[A];
#pragma unroll
  for (int a = 0; a < A; ++a) u[a] = v[b + B * a];
  Dft<A, INV>::run(u);
  ct_twiddle<A, B, INV, b>(u, tmp, std::make_integer_sequence<int, A>{});
}
template <int A, int B, bool INV, int... bs>
__host__ __device__ __forceinline__ void ct_first_all(float2 (&v)[A * B], float2 (&tmp)[A * B], std::integer_sequence<int, bs...>) {
  (ct_first<A, B, INV, bs>(v, tmp), ...);
}
template <int A, int B, bool INV>
__host__ __device__ __forceinline__ void dft_ct(float2 (&v)[A * B]) {
  float2 tmp[A * B];
  ct_first_all<A, B, INV>(v, tmp, std::make_integer_sequence<int, B>{});
#pragma unroll
  for (int ka = 0; ka < A; ++ka) {
    float2 w[B];
#pragma unroll
    for (int b = 0; b < B; ++b) w[b] = tmp[b + B * ka];
    Dft<B, INV>::run(w);
#pragma unroll
    for (int kb = 0; kb < B; ++kb) v[ka + A * kb] = w[kb];
  }
}

template <bool INV> struct Dft<6, INV> {
  static __host__ __device__ __forceinline__ void run(float2 (&v)[6]) { dft_ct<2, 3, INV>(v); }
};
template <bool INV> struct Dft<12, INV> {
  static __host__ __device__ __forceinline__ void run(float2 (&v)[12]) { dft_ct<4, 3, INV>(v); }
};
// 16-point DFT as 4 x 4 (X[ka + 4 kb] over inner DFTs of x[b + 4 a]) with the
// twiddle scales folded into fused multiply-adds.  With s = -1 forward, +1
// inverse, h = cos(pi/4), C = cos(pi/8) and tau = tan(pi/8):
//   W^2 = h (1 + s i), W^4 = s i, W^6 = h (-1 + s i),
//   W^1 = C (1 + s i tau), W^3 = C (tau + s i), W^9 = -C (1 + s i tau),
// so in the outer DFTs of columns ka = 1, 2, 3 the pairs (z1, z3) and z2 carry
// the common scales C and h, which are applied by the butterflies' FMAs:
// 144 operations against 160 with the twiddles multiplied out.
template <bool INV>
__host__ __device__ __forceinline__ void dft16_outer(float2 u0, float2 z2h, float2 q1, float2 q3, float hs, float cs,
                                                     float2& y0, float2& y1, float2& y2, float2& y3) {
  // inputs z0 = u0, z2 = hs * z2h, z1 = cs * q1, z3 = cs * q3; outputs Y_kb of the 4-point DFT
  constexpr float s = INV ? 1.f : -1.f;
  const float2 a = caxpy(hs, z2h, u0);
  const float2 b = caxpy(-hs, z2h, u0);
  const float2 P = cadd(q1, q3), Q = csub(q1, q3);
  y0 = caxpy(cs, P, a);
  y2 = caxpy(-cs, P, a);
  y1 = make_float2(fmaf(-s * cs, Q.y, b.x), fmaf(s * cs, Q.x, b.y));
  y3 = make_float2(fmaf(s * cs, Q.y, b.x), fmaf(-s * cs, Q.x, b.y));
}
// 8-point DFT as 2 x 4: inner 2-point DFTs of x[b], x[b + 4]; the outer DFT of
// the odd outputs has the twiddles W8^1 = h (1 + s i), W8^2 = s i,
// W8^3 = h (-1 + s i), whose common scale h goes into the FMAs (52 operations
// against 56).
template <bool INV> struct Dft<8, INV> {
  static __host__ __device__ __forceinline__ void run(float2 (&v)[8]) {
    constexpr float s = INV ? 1.f : -1.f;
    constexpr float h = 0.70710678118654752440f;
    float2 e[4], o[4];  // inner DFTs: e = x[b] + x[b + 4], o = x[b] - x[b + 4]
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      e[b] = cadd(v[b], v[b + 4]);
      o[b] = csub(v[b], v[b + 4]);
    }
    Dft<4, INV>::run(e);
    const float2 p1 = make_float2(o[1].x - s * o[1].y, o[1].y + s * o[1].x);   // o1 (1 + s i)
    const float2 z2 = make_float2(-s * o[2].y, s * o[2].x);                    // s i o2
    const float2 p3 = make_float2(-o[3].x - s * o[3].y, s * o[3].x - o[3].y);  // o3 (-1 + s i)
    float2 y0, y1, y2, y3;
    dft16_outer<INV>(o[0], z2, p1, p3, 1.f, h, y0, y1, y2, y3);
    v[0] = e[0]; v[2] = e[1]; v[4] = e[2]; v[6] = e[3];
    v[1] = y0; v[3] = y1; v[5] = y2; v[7] = y3;
  }
};
// `odd` (1 or -1) multiplies the odd-indexed inputs: they feed the inner DFTs
// b = 1, 3, i.e. the pairs (z1, z3) of every outer DFT, whose scale it joins.
template <bool INV>
__host__ __device__ __forceinline__ void dft16(float2 (&v)[16], float odd) {
  constexpr float s = INV ? 1.f : -1.f;
  constexpr float h = 0.70710678118654752440f;    // cos(pi/4)
  constexpr float C = 0.92387953251128675613f;    // cos(pi/8)
  constexpr float tau = 0.41421356237309504880f;  // tan(pi/8)
  float2 U[4][4];  // U[b][ka]: inner 4-point DFTs of x[b + 4 a]
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    float2 u[4] = {v[b], v[b + 4], v[b + 8], v[b + 12]};
    Dft<4, INV>::run(u);
#pragma unroll
    for (int k = 0; k < 4; ++k) U[b][k] = u[k];
  }
  const float hodd = h * odd, codd = C * odd;
  // ka = 0: no twiddles
  dft16_outer<INV>(U[0][0], U[2][0], U[1][0], U[3][0], 1.f, odd, v[0], v[4], v[8], v[12]);
  {  // ka = 1: z1 = C q1, z2 = h p2, z3 = C q3
    const float2 u1 = U[1][1], u2 = U[2][1], u3 = U[3][1];
    const float2 q1 = make_float2(fmaf(-s * tau, u1.y, u1.x), fmaf(s * tau, u1.x, u1.y));  // u1 (1 + s i tau)
    const float2 p2 = make_float2(u2.x - s * u2.y, u2.y + s * u2.x);                        // u2 (1 + s i)
    const float2 q3 = make_float2(fmaf(tau, u3.x, -s * u3.y), fmaf(tau, u3.y, s * u3.x));  // u3 (tau + s i)
    dft16_outer<INV>(U[0][1], p2, q1, q3, h, codd, v[1], v[5], v[9], v[13]);
  }
  {  // ka = 2: z1 = h p1, z2 = s i u2, z3 = h p3 (the common scale h goes with z1, z3)
    const float2 u1 = U[1][2], u2 = U[2][2], u3 = U[3][2];
    const float2 p1 = make_float2(u1.x - s * u1.y, u1.y + s * u1.x);   // u1 (1 + s i)
    const float2 z2 = make_float2(-s * u2.y, s * u2.x);                // s i u2
    const float2 p3 = make_float2(-u3.x - s * u3.y, s * u3.x - u3.y);  // u3 (-1 + s i)
    dft16_outer<INV>(U[0][2], z2, p1, p3, 1.f, hodd, v[2], v[6], v[10], v[14]);
  }
  {  // ka = 3: z1 = C q1, z2 = h p2, z3 = C q3
    const float2 u1 = U[1][3], u2 = U[2][3], u3 = U[3][3];
    const float2 q1 = make_float2(fmaf(tau, u1.x, -s * u1.y), fmaf(tau, u1.y, s * u1.x));    // u1 (tau + s i)
    const float2 p2 = make_float2(-u2.x - s * u2.y, s * u2.x - u2.y);                         // u2 (-1 + s i)
    const float2 q3 = make_float2(fmaf(s * tau, u3.y, -u3.x), fmaf(-s * tau, u3.x, -u3.y));  // -u3 (1 + s i tau)
    dft16_outer<INV>(U[0][3], p2, q1, q3, h, codd, v[3], v[7], v[11], v[15]);
  }
}
template <bool INV> struct Dft<16, INV> {
  static __host__ __device__ __forceinline__ void run(float2 (&v)[16]) { dft16<INV>(v, 1.f); }
};
template <bool INV> struct Dft<24, INV> {
  static __host__ __device__ __forceinline__ void run(float2 (&v)[24]) { dft_ct<8, 3, INV>(v); }
};
template <bool INV> struct Dft<32, INV> {
  static __host__ __device__ __forceinline__ void run(float2 (&v)[32]) { dft_ct<4, 8, INV>(v); }
};

// ----------------------------------------------------------------- shared-memory indexers
// Row lines: each line owns a private buffer; one float2 of padding every 32
// keeps the stride-32 writes of a radix-32 stage free of bank conflicts.
struct PaddedLine {
  float2* base;
  __host__ __device__ __forceinline__ float2& operator[](int i) const { return base[i + (i >> 5)]; }
  static constexpr int words(int n) { return n + n / 32; }
};
// Column lines: C columns interleaved element by element (address i*C + c), so
// a warp whose lanes are consecutive columns touches consecutive words.
template <int C>
struct InterleavedLine {
  float2* base;  // already offset by the column
  __host__ __device__ __forceinline__ float2& operator[](int i) const { return base[i * C]; }
};

template <bool CTA>
__device__ __forceinline__ void line_sync() {
  if constexpr (CTA) __syncthreads();
  else __syncwarp();
}

// ----------------------------------------------------------------- Stockham line transform
// Twiddle table layout for a radix list (R1, ..., Rs): stage i (i >= 2) with
// Ns = R1*...*R(i-1) stores W_{Ns Ri}^{k r} at offset_i + (r-1)*Ns + k for
// r = 1..Ri-1, k = 0..Ns-1 (forward sign; the inverse uses the conjugate).
template <int... Rs> struct Radices;

template <int N, int T, class Rad> struct LineFFT;

template <int N, int T, int... Rs>
struct LineFFT<N, T, Radices<Rs...>> {
  using Rad = Radices<Rs...>;
  static constexpr int E = N / T;
  static_assert(N % T == 0, "threads must divide the line");
  static constexpr int kStages = sizeof...(Rs);
  static_assert((Rs * ...) == N, "radices must multiply to the line length");

  static constexpr int tw_words() {
    int ns = 1, total = 0;
    int rs[] = {Rs...};
    for (int i = 0; i < kStages; ++i) { if (i > 0) total += (rs[i] - 1) * ns; ns *= rs[i]; }
    return total;
  }

  // Radix-R butterflies of one Stockham stage for thread t: reads its slots of
  // v, writes the butterfly outputs (slot order q + r*Q) to out.
  template <int R, int Ns, int TwOff, bool INV>
  static __host__ __device__ __forceinline__ void butterflies(const float2 (&v)[E], float2 (&out)[E],
                                                              const float2* __restrict__ tw, int t) {
    static_assert(E % R == 0, "radix must divide the elements per thread");
    constexpr int Q = E / R;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      float2 u[R];
#pragma unroll
      for (int r = 0; r < R; ++r) u[r] = v[q + r * Q];
      if constexpr (Ns > 1) {
        // when Ns divides T every butterfly of the thread uses the same twiddles
        const int k = (T % Ns == 0) ? (t % Ns) : (t + T * q) % Ns;
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const float2 w = tw[TwOff + (r - 1) * Ns + k];
          u[r] = INV ? cmulc(u[r], w) : cmul(u[r], w);
        }
      }
      Dft<R, INV>::run(u);
#pragma unroll
      for (int r = 0; r < R; ++r) out[q + r * Q] = u[r];
    }
  }
  // Stockham destinations of the butterfly outputs of thread t.
  template <int R, int Ns, class Buf>
  static __host__ __device__ __forceinline__ void scatter(const float2 (&out)[E], const Buf& buf, int t) {
    constexpr int Q = E / R;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int j = t + T * q;
      const int idxD = (j / Ns) * Ns * R + (j % Ns);
#pragma unroll
      for (int r = 0; r < R; ++r) buf[idxD + r * Ns] = out[q + r * Q];
    }
  }
  template <class Buf>
  static __host__ __device__ __forceinline__ void gather(float2 (&v)[E], const Buf& buf, int t) {
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = buf[t + T * m];
  }

  // PRESYNC = false skips the synchronisation before this stage's scatter (the
  // caller guarantees that nobody still reads the exchange buffer); later
  // exchanges of the same transform always synchronise.
  template <bool INV, bool CTA, int Ns, int TwOff, bool PRESYNC, class Buf, int R0, int... Rest>
  static __device__ __forceinline__ void stages(float2 (&v)[E], const Buf& buf, const float2* tw, int t) {
    float2 out[E];
    butterflies<R0, Ns, TwOff, INV>(v, out, tw, t);
    if constexpr (sizeof...(Rest) == 0) {
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = out[m];
    } else {
      if constexpr (PRESYNC) line_sync<CTA>();   // previous readers of buf are done
      scatter<R0, Ns>(out, buf, t);
      line_sync<CTA>();
      gather(v, buf, t);
      constexpr int nextOff = (Ns > 1) ? TwOff + (R0 - 1) * Ns : TwOff;
      stages<INV, CTA, Ns * R0, nextOff, true, Buf, Rest...>(v, buf, tw, t);
    }
  }

  // In-place line transform of the E values held by thread t (unnormalised).
  // All T threads of the line must call it together.
  template <bool INV, bool CTA, class Buf, bool PRESYNC = true>
  static __device__ __forceinline__ void run(float2 (&v)[E], const Buf& buf, const float2* tw, int t) {
    stages<INV, CTA, 1, 0, PRESYNC, Buf, Rs...>(v, buf, tw, t);
  }

  // Exchanges alternate between two buffers, b0 for the X0-th exchange of the
  // sequence, b1 for the next, and so on, and no scatter is preceded by a
  // synchronisation: a scatter into one buffer can only race with reads of the
  // same buffer two exchanges earlier, and the synchronisation after the
  // intervening scatter already separates them.  The caller orders the first
  // scatter into each buffer against earlier readers.
  static constexpr int kExchanges = kStages - 1;
  template <bool INV, bool CTA, int Ns, int TwOff, int X, class Buf, int R0, int... Rest>
  static __device__ __forceinline__ void stages_alt(float2 (&v)[E], const Buf& b0, const Buf& b1, const float2* tw,
                                                    int t) {
    float2 out[E];
    butterflies<R0, Ns, TwOff, INV>(v, out, tw, t);
    if constexpr (sizeof...(Rest) == 0) {
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = out[m];
    } else {
      const Buf& buf = (X & 1) ? b1 : b0;
      scatter<R0, Ns>(out, buf, t);
      line_sync<CTA>();
      gather(v, buf, t);
      constexpr int nextOff = (Ns > 1) ? TwOff + (R0 - 1) * Ns : TwOff;
      stages_alt<INV, CTA, Ns * R0, nextOff, X + 1, Buf, Rest...>(v, b0, b1, tw, t);
    }
  }
  template <bool INV, bool CTA, int X0, class Buf>
  static __device__ __forceinline__ void run_alt(float2 (&v)[E], const Buf& b0, const Buf& b1, const float2* tw,
                                                 int t) {
    stages_alt<INV, CTA, 1, 0, X0, Buf, Rs...>(v, b0, b1, tw, t);
  }

  // Host emulation of run() on a whole line (data[N] in natural order), used
  // by the host-side unit test of the index arithmetic and the codelets.
  template <bool INV, int Ns, int TwOff, int R0, int... Rest>
  static void host_stages(float2 (*v)[E], float2* scratch, const float2* tw) {
    float2 out[T][E];
    for (int t = 0; t < T; ++t) butterflies<R0, Ns, TwOff, INV>(v[t], out[t], tw, t);
    if constexpr (sizeof...(Rest) == 0) {
      for (int t = 0; t < T; ++t) for (int m = 0; m < E; ++m) v[t][m] = out[t][m];
    } else {
      PaddedLine buf{scratch};
      for (int t = 0; t < T; ++t) scatter<R0, Ns>(out[t], buf, t);
      for (int t = 0; t < T; ++t) gather(v[t], buf, t);
      constexpr int nextOff = (Ns > 1) ? TwOff + (R0 - 1) * Ns : TwOff;
      host_stages<INV, Ns * R0, nextOff, Rest...>(v, scratch, tw);
    }
  }
  template <bool INV>
  static void host_run(float2* data, const float2* tw) {
    static float2 v[T][E];
    static float2 scratch[PaddedLine::words(N)];
    for (int t = 0; t < T; ++t) for (int m = 0; m < E; ++m) v[t][m] = data[t + T * m];
    host_stages<INV, 1, 0, Rs...>(v, scratch, tw);
    for (int t = 0; t < T; ++t) for (int m = 0; m < E; ++m) data[t + T * m] = v[t][m];
  }
  // Inter-stage twiddle table in the layout documented above (forward sign).
  static void host_twiddles(float2* tw) {
    int rs[] = {Rs...};
    int ns = 1, off = 0;
    for (int i = 0; i < kStages; ++i) {
      if (i > 0) {
        for (int r = 1; r < rs[i]; ++r)
          for (int k = 0; k < ns; ++k) {
            long num = (long)k * r, den = (long)ns * rs[i];
            tw[off + (r - 1) * ns + k] = make_float2((float)ce_trig2pi(num, den, false),
                                                     -(float)ce_trig2pi(num, den, true));
          }
        off += (rs[i] - 1) * ns;
      }
      ns *= rs[i];
    }
  }
};

// ----------------------------------------------------------------- paired radix-2 line transform
// Lines of 512 held by one warp (32 threads x 16 values, thread t holding
// elements t + 32 m) with the radices (16, 2, 16) of LineFFT and its twiddle
// table, but with the radix-2 stage done across lane pairs instead of through
// shared memory.  After the first radix-16 stage, the Stockham butterfly
// j = 16 t' + r (t' < 16) of the radix-2 stage combines output r of lane t'
// (value a) with output r of lane t' + 16 (value b), and its twiddle W_32^r
// depends on r alone.  Lane t' computes the butterflies r < 8, lane t' + 16
// those with r >= 8, and each sends the other the eight values it needs (two
// 32-bit shuffles apiece).  So that both lanes send the same register, the
// upper lane negates its odd inputs, which moves output (r + 8) mod 16 of its
// radix-16 DFT into register r: lane t' then sends a[8 + I] and lane t' + 16
// sends b[I] from register 8 + I.  Butterfly outputs y0 = a + W b and
// y1 = a - W b land at 32 t' + r and 32 t' + 16 + r; the last stage reads
// t + 32 m.  Bank-conflict-free through the swizzle p ^ ((p >> 5) & 15): a
// store of one register by a half warp covers 32 t' + c for sixteen t' and one
// c < 32, a load 32 m + t for sixteen consecutive t.  One exchange through
// shared memory per transform instead of two.
__device__ __forceinline__ void sts64(unsigned addr, float2 v) {
  asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ float2 lds64(unsigned addr) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr) : "memory");
  return v;
}

struct PairedFFT512 {
  static constexpr int N = 512, T = 32, E = 16;
  using Base = LineFFT<512, 32, Radices<16, 2, 16>>;
  static constexpr int kStage2Tw = 16;  // offset of the last stage's twiddles in Base's table
  struct Line {
    float2* base;
    __host__ __device__ __forceinline__ float2& operator[](int i) const { return base[i ^ ((i >> 5) & 15)]; }
  };
  // first radix-16 stage of thread t (upper lane: h = t >= 16, odd inputs negated)
  template <bool INV>
  static __host__ __device__ __forceinline__ void first(float2 (&v)[E], bool h) {
    dft16<INV>(v, h ? -1.f : 1.f);
  }
  // radix-2 butterfly I (< 8) of this lane; `recv` is the partner's register 8 + I.
  // W_32^I = (c, s sn) is applied as a scale times (1 + i s t) or (t + i s)
  // with t <= 1, the scale going into the butterfly's FMAs.
  template <bool INV, int I>
  static __host__ __device__ __forceinline__ void pair(float2 (&v)[E], float2 recv, bool h) {
    constexpr float s = INV ? 1.f : -1.f;
    constexpr double cw = ce_trig2pi(I, 32, false), sw = ce_trig2pi(I, 32, true);
    constexpr bool by_cos = cw >= sw;
    constexpr float scale = (float)(by_cos ? cw : sw);
    constexpr float t = (float)(by_cos ? sw / cw : cw / sw);
    const float2 a = h ? recv : v[I];
    const float2 b = h ? v[I] : recv;
    float2 q;
    if constexpr (I == 0) q = b;
    else if constexpr (by_cos) q = make_float2(fmaf(-s * t, b.y, b.x), fmaf(s * t, b.x, b.y));  // b (1 + i s t)
    else q = make_float2(fmaf(t, b.x, -s * b.y), fmaf(t, b.y, s * b.x));                         // b (t + i s)
    const float2 q8 = make_float2(-s * q.y, s * q.x);  // the upper lane's butterfly is I + 8: times W_32^8 = s i
    q = h ? q8 : q;
    v[I] = make_float2(fmaf(scale, q.x, a.x), fmaf(scale, q.y, a.y));
    v[8 + I] = make_float2(fmaf(-scale, q.x, a.x), fmaf(-scale, q.y, a.y));
  }
  // line position of register m of thread t after the radix-2 stage
  static __host__ __device__ __forceinline__ int pos(int m, int t) {
    return 32 * (t & 15) + 8 * (t >> 4) + m + (m >= 8 ? 8 : 0);
  }
  // The same exchange as byte offsets in a 256-byte-aligned line, in a form
  // with one logic operation per access: the store of register m is
  // st_base(t) ^ 8 c_m (c_m = m + 8 [m >= 8]) and the load of element
  // t + 32 m is ((8 t) ^ (8 m)) + 256 m, both equal to 8 Line-index.
  static __host__ __device__ __forceinline__ unsigned st_base(int t) {
    return 256u * (t & 15) + 8u * ((8 * (t >> 4)) ^ (t & 15));
  }
  static __host__ __device__ __forceinline__ unsigned st_off(int m, int t) {
    return st_base(t) ^ (8u * (m + (m >= 8 ? 8 : 0)));
  }
  static __host__ __device__ __forceinline__ unsigned ld_off(int m, int t) {
    return ((8u * t) ^ (8u * m)) + 256u * m;
  }
  template <bool INV, int... Is>
  static __device__ __forceinline__ void pairs(float2 (&v)[E], bool h, std::integer_sequence<int, Is...>) {
    (pair<INV, Is>(v, make_float2(__shfl_xor_sync(0xffffffffu, v[8 + Is].x, 16),
                                  __shfl_xor_sync(0xffffffffu, v[8 + Is].y, 16)), h), ...);
  }
  // In-place transform of the line held by the warp (unnormalised); `line` is
  // the shared-memory address of the warp's 512-word exchange buffer, 256-byte
  // aligned, whose earlier readers must be this warp's own threads.
  template <bool INV>
  static __device__ __forceinline__ void run(float2 (&v)[E], unsigned line, const float2* tw, int t) {
    const bool h = t >= 16;
    first<INV>(v, h);
    pairs<INV>(v, h, std::make_integer_sequence<int, 8>{});
    __syncwarp();  // earlier reads of the buffer are done
    const unsigned q = line + st_base(t);
#pragma unroll
    for (int m = 0; m < E; ++m) sts64(q ^ (8u * (m + (m >= 8 ? 8 : 0))), v[m]);
    __syncwarp();
    const unsigned r = line + 8u * t;
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = lds64((r ^ (8u * m)) + 256u * m);
    float2 out[E];
    Base::template butterflies<16, 32, kStage2Tw, INV>(v, out, tw, t);
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = out[m];
  }

  // Host emulation of run() on a whole line (natural order), for the host-side
  // check of the lane arithmetic; the shuffles become reads of the partner's
  // registers.
  template <bool INV, int... Is>
  static void host_pairs(float2 (*v)[E], std::integer_sequence<int, Is...>) {
    auto one = [&](auto ic) {
      constexpr int I = decltype(ic)::value;
      float2 recv[T];
      for (int t = 0; t < T; ++t) recv[t] = v[t ^ 16][8 + I];
      for (int t = 0; t < T; ++t) pair<INV, I>(v[t], recv[t], t >= 16);
    };
    (one(std::integral_constant<int, Is>{}), ...);
  }
  template <bool INV>
  static void host_run(float2* data, const float2* tw) {
    static float2 v[T][E];
    static float2 scratch[N];
    const Line buf{scratch};
    for (int t = 0; t < T; ++t) for (int m = 0; m < E; ++m) v[t][m] = data[t + T * m];
    for (int t = 0; t < T; ++t) first<INV>(v[t], t >= 16);
    host_pairs<INV>(v, std::make_integer_sequence<int, 8>{});
    for (int t = 0; t < T; ++t) for (int m = 0; m < E; ++m) buf[pos(m, t)] = v[t][m];
    for (int t = 0; t < T; ++t) {
      for (int m = 0; m < E; ++m) v[t][m] = buf[t + T * m];
      float2 out[E];
      Base::template butterflies<16, 32, kStage2Tw, INV>(v[t], out, tw, t);
      for (int m = 0; m < E; ++m) data[t + T * m] = out[m];
    }
  }
  static constexpr int tw_words() { return Base::tw_words(); }
  static void host_twiddles(float2* tw) { Base::host_twiddles(tw); }
};

}  // namespace msx
