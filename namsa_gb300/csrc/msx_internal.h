// Internal declarations shared by the translation units of libmsx.so.
#pragma once
#include <cuda_runtime.h>

#include "msx_sched.cuh"

namespace msx {

cudaError_t launch_atom_windows(const double* coeff, int nspecies, int n0, int n1, int os, double range, float* out,
                                cudaStream_t st);
cudaError_t launch_potential(const int4* sites, const int* slice_off, int num_slices, const float* windows, int H, int W,
                             int Ny, int Nx, float sigma, float2* trans, float* pot, cudaStream_t st);
cudaError_t launch_probe(int Ny, int Nx, float kmax, double lambda, float k_semi, double C1, double C3, double C5,
                         int smooth, float2* psik, float* aperture, double* norm, cudaStream_t st);
// *dst = value, as a one-thread kernel on st.
cudaError_t launch_store_double(double* dst, double value, cudaStream_t st);
// Sets the message returned by msx_last_error for the calling thread.
void set_last_error(const char* msg);

cudaError_t launch_detect_reduce(const float* partial, int G, int tiles, int ndet, float* out, cudaStream_t st);
cudaError_t launch_pfac(int Ny, int Nx, float kmax, double lambda, double slice_t, float k_band, float2* pyx,
                        int2* band, cudaStream_t st);
cudaError_t launch_ptab(int Ny, int Nx, float kmax, double lambda, double slice_t, float k_band, float2* ptab,
                        cudaStream_t st);

// Strided addressing of a matrix element (r, k):
//   (r / rc) * s1 + (r % rc) * s2 + (k / kc) * t1 + (k % kc) * t2.
struct Addr {
  long long s1, s2, rc;
  long long t1, t2, kc;
};
// Row-major with leading dimension ld.
inline Addr rowmajor(long long ld) { return Addr{ld, 0, 1, 1, 0, 1}; }
// Element (r, k) at r + k * ld (column-major / transposed operand).
inline Addr colmajor(long long ld) { return Addr{1, 0, 1, ld, 0, 1}; }

// Epilogue of the tensor-core GEMM: z = scale * acc (+ bias[c]) (+ add[o]) (+ y[o] when accumulate);
// y[o] = z; act[o] = gelu(z) when act is set; o is the address of (r, c) under `out`.
struct Epi {
  float* y;
  Addr out;
  long long M;
  int N;
  const float* bias;
  const float* add;
  float* act;
  int accumulate;
  float scale;
  long long ybs;  // batched GEMMs: offset of batch b's output (y, add, act) is b * ybs
};

// D (M x N) = A (M x K) . B (N x K)^T on tcgen05 in bfloat16 with FP32 accumulation
// (msx_tcgemm.cu).  Operand images and the error word are owned by the object.
struct TcGemm {
  void* a_img = nullptr;
  void* b_img = nullptr;
  size_t a_cap = 0, b_cap = 0;
  int* err = nullptr;
  int reserve(size_t a_bytes, size_t b_bytes);
  float* part = nullptr;  // split-K partial sums
  size_t part_cap = 0;
  // ksplit > 1 splits K (for the long-K weight gradients): with N <= 32 over
  // max(ksplit, one per resident CTA) splits of the persistent kernel, both operands
  // staged from FP32; otherwise over ksplit CTAs per tile with packed operands.
  // Partial tiles are summed in a fixed order before the epilogue.
  int run(const float* a, Addr aa, const float* b, Addr ba, long long M, int N, long long K, const Epi& e,
          cudaStream_t st, int ksplit = 1);
  // `batch` independent GEMMs of the same shape; batch b reads A at a + b * a_bs, B at
  // b_ptr + b * b_bs and writes at e.y + b * y_bs (floats); no K split.
  int run_batched(const float* a, Addr aa, long long a_bs, const float* b, Addr ba, long long b_bs, long long M,
                  int N, long long K, const Epi& e, long long y_bs, int batch, cudaStream_t st);
  // `batch` complex products in one real GEMM each: B (2 hn x 2 hk) is the real
  // embedding of src (pack_cplx_kernel: element (i, j) at src + i si + j sj, parts
  // interleaved, negated block neg = 1 for (0, 1), 2 for (1, 0)); src of batch b at
  // src + b * src_bs.
  int run_cplx(const float* a, Addr aa, long long a_bs, const float* src, long long si, long long sj,
               long long src_bs, int hn, int hk, int neg, long long M, const Epi& e, long long y_bs, int batch,
               cudaStream_t st);
  int check();
  void release();
};

}  // namespace msx
