// msx_multislice_noalloc: the multislice of msx_multislice for callers that
// cannot allocate device memory.  Its scratch (twiddle tables, propagator
// table and the resident wave group) lives in one file-scope __device__ array
// of fixed size instead of a plan's cudaMalloc'd workspace.
#include "msx.h"
#include "msx_internal.h"

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

using namespace msx;

namespace {

// 32 MiB of complex64 words, held by every device that loads the library until
// the process exits.
constexpr size_t kScratchWords = (size_t)4 << 20;
constexpr size_t kTwWords = 1024;  // per twiddle table (largest schedule-0 table: 992 words)

static __device__ __align__(256) float2 g_scratch[kScratchWords];

// Host-side cache of the scratch's device address, one per device.  The name
// g_scratch in host code is only a host-side stand-in; the device address
// comes from cudaGetSymbolAddress with that device current.  The mutex makes
// the first call on a device safe from several host threads at once.
constexpr int kMaxDev = 64;
float2* g_scratch_dev[kMaxDev];
bool g_scratch_ready[kMaxDev];
std::mutex g_scratch_mutex;

bool aligned_to(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  set_last_error(buf);  // read back through msx_last_error
  return code;
}

// Radices of schedule 0 of each line length (csrc/msx_pass_<N>.cu).
struct Rad { int n, count, r[4]; };
constexpr Rad kRad[] = {{64, 2, {8, 8}},       {128, 2, {16, 8}},     {256, 2, {16, 16}}, {384, 3, {8, 8, 6}},
                        {512, 2, {32, 16}},    {768, 3, {8, 8, 12}},  {1024, 2, {32, 32}}};

const Rad* radices_of(int n) {
  for (const Rad& r : kRad)
    if (r.n == n) return &r;
  return nullptr;
}

int tw_words_of(const Rad& rd) {
  int ns = 1, total = 0;
  for (int i = 0; i < rd.count; ++i) { if (i > 0) total += (rd.r[i] - 1) * ns; ns *= rd.r[i]; }
  return total;
}

// Inter-stage twiddles in the layout of LineFFT (msx_fft.cuh): stage i >= 1 with
// Ns = R0*...*R(i-1) holds exp(-2 pi i k r / (Ns Ri)) at offset_i + (r-1)*Ns + k.
__global__ void twiddle_fill_kernel(Rad rd, float2* __restrict__ tw) {
  int ns = 1, off = 0;
  for (int i = 0; i < rd.count; ++i) {
    if (i > 0) {
      const int R = rd.r[i], cnt = (R - 1) * ns;
      for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
        const int r = 1 + e / ns, k = e % ns;
        const long long den = (long long)ns * R;
        const long long num = ((long long)k * r) % den;
        double s, c;
        sincospi(-2.0 * (double)num / (double)den, &s, &c);
        tw[off + e] = make_float2((float)c, (float)s);
      }
      off += (R - 1) * ns;
    }
    ns *= rd.r[i];
  }
}

int ensure_scratch(int dev, float2** out) {
  if (dev < 0 || dev >= kMaxDev) return fail(MSX_ERR_INVALID, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ready[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return fail(MSX_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_scratch_dev[dev] = static_cast<float2*>(p);
    g_scratch_ready[dev] = true;
  }
  *out = g_scratch_dev[dev];
  return MSX_OK;
}

}  // namespace

extern "C" MSX_API int msx_multislice_noalloc(const float* trans_dev, int num_slices, const float* psi_k_dev,
                                              const double* normalization_dev, const float* positions_dev,
                                              int num_probes, int ny, int nx, float kmax, double lambda,
                                              double slice_t, float k_band, float* cbed_out_dev, int crop_y,
                                              int crop_x, void* stream) {
  if (ny <= 0 || nx <= 0) return fail(MSX_ERR_INVALID, "bad grid %d x %d", ny, nx);
  const size_t wave = (size_t)ny * nx;
  const size_t fixed = 2 * kTwWords + wave;
  if (fixed + wave > kScratchWords)
    return fail(MSX_ERR_INVALID, "grid %d x %d needs %zu bytes of scratch; the static scratch holds %zu bytes",
                ny, nx, sizeof(float2) * (fixed + wave), sizeof(float2) * kScratchWords);
  const Rad* rr = radices_of(nx);
  const Rad* rc = radices_of(ny);
  if (!rr || !rc)
    return fail(MSX_ERR_UNSUPPORTED, "grid %d x %d: supported line lengths are 64, 128, 256, 384, 512, 768, 1024", ny, nx);
  if (num_probes < 0 || num_slices < 0) return fail(MSX_ERR_INVALID, "negative probe or slice count");
  if (num_probes == 0) return MSX_OK;
  if (crop_y <= 0 || crop_x <= 0 || crop_y > ny || crop_x > nx)
    return fail(MSX_ERR_INVALID, "crop %d x %d outside the %d x %d grid", crop_y, crop_x, ny, nx);
  if (!psi_k_dev || !normalization_dev || !positions_dev || !cbed_out_dev || (num_slices > 0 && !trans_dev))
    return fail(MSX_ERR_INVALID, "null pointer");
  if (!aligned_to(trans_dev, 8) || !aligned_to(psi_k_dev, 8) || !aligned_to(positions_dev, 8) ||
      !aligned_to(normalization_dev, 8) || !aligned_to(cbed_out_dev, 4))
    return fail(MSX_ERR_INVALID, "complex inputs, positions and the normalisation must be 8-byte aligned, "
                "the output 4-byte aligned");
  if (!(kmax > 0) || !(lambda > 0) || !(slice_t >= 0) || !(k_band >= 0))
    return fail(MSX_ERR_INVALID, "kmax, lambda must be positive; slice thickness and k_band non-negative");
  size_t g = (kScratchWords - fixed) / wave;
  if (g > (size_t)num_probes) g = (size_t)num_probes;
  const int group = (int)g;

  const SchedOps *rops, *cops;
  int n_r = 0, n_c = 0;
  switch (nx) {
    case 64: n_r = schedules_64(&rops); break; case 128: n_r = schedules_128(&rops); break;
    case 256: n_r = schedules_256(&rops); break; case 384: n_r = schedules_384(&rops); break;
    case 512: n_r = schedules_512(&rops); break; case 768: n_r = schedules_768(&rops); break;
    default: n_r = schedules_1024(&rops); break;
  }
  switch (ny) {
    case 64: n_c = schedules_64(&cops); break; case 128: n_c = schedules_128(&cops); break;
    case 256: n_c = schedules_256(&cops); break; case 384: n_c = schedules_384(&cops); break;
    case 512: n_c = schedules_512(&cops); break; case 768: n_c = schedules_768(&cops); break;
    default: n_c = schedules_1024(&cops); break;
  }
  if (n_r < 1 || n_c < 1 || rops[0].tw_words != tw_words_of(*rr) || cops[0].tw_words != tw_words_of(*rc))
    return fail(MSX_ERR_INVALID, "schedule tables disagree with the static twiddle layout");
  const SchedOps& row = rops[0];
  const SchedOps& col = cops[0];

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(MSX_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  float2* base = nullptr;
  int rc_ = ensure_scratch(dev, &base);
  if (rc_ != MSX_OK) return rc_;
  e = row.configure();
  if (e == cudaSuccess) e = col.configure();
  if (e != cudaSuccess) return fail(MSX_ERR_CUDA, "configuring pass kernels: %s", cudaGetErrorString(e));

  float2* tw_row = base;
  float2* tw_col = base + kTwWords;
  float2* ptab = base + 2 * kTwWords;
  float2* psi = ptab + wave;
  cudaStream_t st = (cudaStream_t)stream;
#define NA_CUDA(call, what)                                                                         \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return fail(MSX_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e_));       \
  } while (0)
  twiddle_fill_kernel<<<1, 256, 0, st>>>(*rr, tw_row);
  NA_CUDA(cudaGetLastError(), "twiddle table");
  twiddle_fill_kernel<<<1, 256, 0, st>>>(*rc, tw_col);
  NA_CUDA(cudaGetLastError(), "twiddle table");
  NA_CUDA(launch_ptab(ny, nx, kmax, lambda, slice_t, k_band, ptab, st), "propagator table");
  const int y0 = ny / 2 - crop_y / 2, x0 = nx / 2 - crop_x / 2;
  const float2* trans = reinterpret_cast<const float2*>(trans_dev);
  for (int g0 = 0; g0 < num_probes; g0 += group) {
    const int gn = (num_probes - g0 < group) ? num_probes - g0 : group;
    ColArgs c{};
    c.psi = psi;
    c.ptab = ptab;
    c.psik = reinterpret_cast<const float2*>(psi_k_dev);
    c.pos_yx = positions_dev + 2 * (size_t)g0;
    c.tw = tw_col;
    c.norm = normalization_dev;
    c.cbed = cbed_out_dev + (size_t)g0 * crop_y * crop_x;
    c.G = gn;
    c.Nx = nx;
    c.kmax = kmax;
    c.y0 = y0;
    c.crop_y = crop_y;
    if (num_slices == 0) {
      c.x_begin = x0;
      c.ncols = crop_x;
      NA_CUDA(col.col(COL_INIT_FINAL, c, st), "probe-only pass");
      continue;
    }
    c.x_begin = 0;
    c.ncols = nx;
    NA_CUDA(col.col(COL_INIT, c, st), "probe formation pass");
    for (int s = 0; s < num_slices; ++s) {
      NA_CUDA(row.row(psi, trans + (size_t)s * wave, tw_row, gn, ny, st), "row pass");
      if (s + 1 < num_slices) {
        NA_CUDA(col.col(COL_MID, c, st), "column pass");
      } else {
        ColArgs f = c;
        f.x_begin = x0;
        f.ncols = crop_x;
        NA_CUDA(col.col(COL_FINAL, f, st), "final column pass");
      }
    }
  }
#undef NA_CUDA
  return MSX_OK;
}
